// rtm_kernels.cu -- sm_103a kernels of the RTM engine.
//
//   k_step   one fused time step: 8th-order leapfrog (SRC/stencilDFM.c:7-31), CPML
//            corrections (SRC/absorbingBoundaryCondition.c:191-357), source injection
//            (SRC/forward_modeling.c:105-109) or receiver overwrite
//            (SRC/backward_modeling.c:277-281), trace recording, boundary-ring or
//            snapshot storage, reverse-time source reconstruction and the FP64
//            cross-correlation image (SRC/image_conditions.c:20-33).
//   k_psi    CPML psi update of the four strips (absorbingBoundaryCondition.c:171-189,
//            219-235, 265-281, 312-328); runs before k_step each step.
//   others   set-up (coef), seismogram transpose, image/field layout conversion, the
//            post-stack Laplacian (SRC/math_functions.c:9-27).
//
// The wavefield tile is loaded by TMA (cp.async.bulk.tensor.2d) into shared memory with
// a 4-cell halo; each thread keeps a 9-column register window along x and reads its z
// neighbours as aligned 16-byte vectors from the tile row.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "rtm_internal.h"

namespace rtm {

// 8th-order second-derivative weights (SRC/stencilDFM.h:8-12)
#define RTM_AC0 (-2.97399944f)
#define RTM_AC1 (+1.70507669f)
#define RTM_AC2 (-0.25861812f)
#define RTM_AC3 (+0.04577745f)
#define RTM_AC4 (-0.00523630f)
// 8th-order first-derivative weights (SRC/absorbingBoundaryCondition.h:21-24)
#define RTM_B1 (+0.8f)
#define RTM_B2 (-0.2f)
#define RTM_B3 (+0.025396825f)
#define RTM_B4 (-0.001785714f)

// Scale targets of 16-bit storage: the tile's max |u| is stored as this value.
constexpr float kFp16Target = 16384.0f;
constexpr float kBf16Target = 1.0f;

// ---- PTX helpers -------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
}

__device__ __forceinline__ void fence_barrier_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int c0, int c1,
                                            uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Bounded wait on an mbarrier phase: gives up after `limit_ns` nanoseconds.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity,
                                                  uint64_t limit_ns)
{
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    while (!mbar_try_wait(bar, parity)) {
        if (global_ns() - t0 > limit_ns) return false;
    }
    return true;
}

// ---- 4-wide vector helpers (16 B for float, 2 x 16 B for double) -------------------------
__device__ __forceinline__ void ld4(const float *p, float (&q)[4])
{
    const float4 v = *reinterpret_cast<const float4 *>(p);
    q[0] = v.x; q[1] = v.y; q[2] = v.z; q[3] = v.w;
}
__device__ __forceinline__ void ld4(const double *p, double (&q)[4])
{
    const double2 a = reinterpret_cast<const double2 *>(p)[0];
    const double2 b = reinterpret_cast<const double2 *>(p)[1];
    q[0] = a.x; q[1] = a.y; q[2] = b.x; q[3] = b.y;
}
__device__ __forceinline__ void ldg4(const float *p, float (&q)[4])
{
    const float4 v = __ldg(reinterpret_cast<const float4 *>(p));
    q[0] = v.x; q[1] = v.y; q[2] = v.z; q[3] = v.w;
}
__device__ __forceinline__ void ldg4(const double *p, double (&q)[4])
{
    const double2 a = __ldg(reinterpret_cast<const double2 *>(p));
    const double2 b = __ldg(reinterpret_cast<const double2 *>(p) + 1);
    q[0] = a.x; q[1] = a.y; q[2] = b.x; q[3] = b.y;
}
__device__ __forceinline__ void st4(float *p, const float (&q)[4])
{
    *reinterpret_cast<float4 *>(p) = make_float4(q[0], q[1], q[2], q[3]);
}
__device__ __forceinline__ void st4(double *p, const double (&q)[4])
{
    reinterpret_cast<double2 *>(p)[0] = make_double2(q[0], q[1]);
    reinterpret_cast<double2 *>(p)[1] = make_double2(q[2], q[3]);
}

// ---- geometry predicates -----------------------------------------------------------------
// Index of cell (x,z) in the boundary ring that encloses the reconstruction region
// [rx0,rx1) x [rz0,rz1) with a 4-cell band, or -1.  Bands: top (x-major, 4 z each),
// bottom, left (4 columns of rz1-rz0), right.
__device__ __forceinline__ int ring_index(const Geom &g, int x, int z)
{
    if (x < g.rx0 - 4 || x >= g.rx1 + 4 || z < g.rz0 - 4 || z >= g.rz1 + 4) return -1;
    if (z < g.rz0) return (x - (g.rx0 - 4)) * 4 + (z - (g.rz0 - 4));
    if (z >= g.rz1) return g.ring_w * 4 + (x - (g.rx0 - 4)) * 4 + (z - g.rz1);
    if (x < g.rx0) return g.ring_w * 8 + (x - (g.rx0 - 4)) * g.ring_h + (z - g.rz0);
    if (x >= g.rx1) return g.ring_w * 8 + 4 * g.ring_h + (x - g.rx1) * g.ring_h + (z - g.rz0);
    return -1;
}

__device__ __forceinline__ bool in_region(const Geom &g, int x, int z)
{
    return x >= g.rx0 && x < g.rx1 && z >= g.rz0 && z < g.rz1;
}

__device__ __forceinline__ bool in_interior(const Geom &g, int x, int z)
{
    return x >= g.thl && x < g.thl + g.nx && z >= g.thu && z < g.thu + g.nz;
}

// Stored source-wavefield element: full precision (T) or 16-bit with a tile scale.
template <typename T>
__device__ __forceinline__ void store_put(void *base, int prec, size_t i, T v, float inv_scale)
{
    if (prec == 1)
        reinterpret_cast<__nv_bfloat16 *>(base)[i] = __float2bfloat16_rn((float)v * inv_scale);
    else if (prec == 2)
        reinterpret_cast<__half *>(base)[i] = __float2half_rn((float)v * inv_scale);
    else
        reinterpret_cast<T *>(base)[i] = v;
}

template <typename T>
__device__ __forceinline__ T store_get(const void *base, int prec, size_t i, float scale)
{
    if (prec == 1)
        return (T)(__bfloat162float(reinterpret_cast<const __nv_bfloat16 *>(base)[i]) * scale);
    if (prec == 2) return (T)(__half2float(reinterpret_cast<const __half *>(base)[i]) * scale);
    return reinterpret_cast<const T *>(base)[i];
}

// Laplacian of the 4 cells of a quad, from the 9-column window W (x) and the 12-value z
// line zz (zm | centre | zp).  Operand order as SRC/stencilDFM.c:24-28.
template <typename T>
__device__ __forceinline__ T lap8(const T (&W)[9][4], const T (&zz)[12], int j)
{
    const T c0 = (T)2.0f * (T)RTM_AC0;
    return c0 * W[4][j]
        + (T)RTM_AC1 * (((W[3][j] + W[5][j]) + zz[3 + j]) + zz[5 + j])
        + (T)RTM_AC2 * (((W[2][j] + W[6][j]) + zz[2 + j]) + zz[6 + j])
        + (T)RTM_AC3 * (((W[1][j] + W[7][j]) + zz[1 + j]) + zz[7 + j])
        + (T)RTM_AC4 * (((W[0][j] + W[8][j]) + zz[0 + j]) + zz[8 + j]);
}

// First derivative along a strided line (B coefficients, :183-186 order).
template <typename T>
__device__ __forceinline__ T d1(const T *f, ptrdiff_t s)
{
    return (T)RTM_B4 * (f[4 * s] - f[-4 * s]) + (T)RTM_B3 * (f[3 * s] - f[-3 * s])
         + (T)RTM_B2 * (f[2 * s] - f[-2 * s]) + (T)RTM_B1 * (f[s] - f[-s]);
}

template <int WARPS>
__device__ __forceinline__ float block_max(float v, float *red)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    float m = red[0];
#pragma unroll
    for (int w = 1; w < WARPS; ++w) m = fmaxf(m, red[w]);
    __syncthreads();
    return m;
}

#include "rtm_step.cuh"

// ---- CPML psi update (runs before k_step) -------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) k_psi(const PsiArgs<T> a)
{
    const Geom &g = a.g;
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    const size_t P = (size_t)g.pitch;
    switch (blockIdx.y) {
    case 0: {   // left strip, x in [4, thl-4), z in [4, dimz-4)
        const int w = g.dimz - 8;
        if (idx >= (g.thl - 8) * w) return;
        const int x = 4 + idx / w, z = 4 + idx % w;
        const size_t at = (size_t)x * P + z;
        a.psi_l[at] = (T)a.b_l[x] * a.psi_l[at] + (T)a.a_l[x] * d1<T>(a.u + at, (ptrdiff_t)P) * a.h1;
        break;
    }
    case 1: {   // top strip, x in [4, dimx-4), z in [4, thu-4)
        const int w = g.thu - 8;
        if (idx >= (g.dimx - 8) * w) return;
        const int x = 4 + idx / w, z = 4 + idx % w;
        const size_t ap = (size_t)x * g.st + z;
        a.psi_t[ap] = (T)a.b_t[z] * a.psi_t[ap] + (T)a.a_t[z] * d1<T>(a.u + (size_t)x * P + z, 1) * a.h1;
        break;
    }
    case 2: {   // right strip, x in [dimx-thr+4, dimx-4)
        const int w = g.dimz - 8;
        if (idx >= (g.thr - 8) * w) return;
        const int li = 4 + idx / w, z = 4 + idx % w;
        const int x = g.dimx - g.thr + li;
        const size_t ap = (size_t)li * P + z;
        a.psi_r[ap] = (T)a.b_r[li] * a.psi_r[ap] +
                      (T)a.a_r[li] * d1<T>(a.u + (size_t)x * P + z, (ptrdiff_t)P) * a.h1;
        break;
    }
    default: {  // bottom strip, z in [dimz-thd+4, dimz-4)
        const int w = g.thd - 8;
        if (idx >= (g.dimx - 8) * w) return;
        const int x = 4 + idx / w, lz = 4 + idx % w;
        const int z = g.dimz - g.thd + lz;
        const size_t ap = (size_t)x * g.sb + lz;
        a.psi_b[ap] = (T)a.b_b[lz] * a.psi_b[ap] +
                      (T)a.a_b[lz] * d1<T>(a.u + (size_t)x * P + z, 1) * a.h1;
        break;
    }
    }
}

// ---- set-up and layout kernels ------------------------------------------------------------
template <typename T>
__global__ void k_coef(Geom g, const float *vel, int vel_pitch, T *coef, float dx, float dt)
{
    const int z = blockIdx.x * blockDim.x + threadIdx.x;
    const int x = blockIdx.y;
    if (z >= g.pitch || x >= g.dimx) return;
    T c = (T)0;
    if (z < g.dimz) {
        // SRC/forward_modeling.c:71-79: coef = (v*dt/dx)^2, dt/dx rounded in T
        const T ratio = (T)dt / (T)dx;
        const T s = (T)vel[(size_t)x * vel_pitch + z] * ratio;
        c = s * s;
    }
    coef[(size_t)x * g.pitch + z] = c;
}

__global__ void k_transpose(const float *in, float *out, int rows, int cols)
{
    __shared__ float tile[32][33];
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int r = r0 + i, c = c0 + threadIdx.x;
        if (r < rows && c < cols) tile[i][threadIdx.x] = in[(size_t)r * cols + c];
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int c = c0 + i, r = r0 + threadIdx.x;
        if (r < rows && c < cols) out[(size_t)c * rows + r] = tile[threadIdx.x][i];
    }
}

template <typename T>
__global__ void k_image_out(Geom g, const double *img, T *out, int accumulate)
{
    const int z = blockIdx.x * blockDim.x + threadIdx.x;
    const int x = blockIdx.y;
    if (z >= g.nz || x >= g.nx) return;
    const double v = img[(size_t)x * g.pitch + g.thu + z];
    T *o = out + (size_t)x * g.nz + z;
    *o = accumulate ? (T)((double)*o + v) : (T)v;
}

template <typename T>
__global__ void k_field_out(Geom g, const T *field, T *out)
{
    const int z = blockIdx.x * blockDim.x + threadIdx.x;
    const int x = blockIdx.y;
    if (z >= g.dimz || x >= g.dimx) return;
    out[(size_t)x * g.dimz + z] = field[(size_t)x * g.pitch + z];
}

template <typename T>
__global__ void k_field_in(Geom g, const T *in, T *field)
{
    const int z = blockIdx.x * blockDim.x + threadIdx.x;
    const int x = blockIdx.y;
    if (z >= g.pitch || x >= g.dimx) return;
    field[(size_t)x * g.pitch + z] = z < g.dimz ? in[(size_t)x * g.dimz + z] : (T)0;
}

// SRC/math_functions.c:9-27: 8th-order Laplacian without 1/dx^2 on [4,nx-4) x [4,nz-4)
__global__ void k_laplacian(int nx, int nz, const float *in, float *out)
{
    const int z = blockIdx.x * blockDim.x + threadIdx.x;
    const int x = blockIdx.y;
    if (x < 4 || x >= nx - 4 || z < 4 || z >= nz - 4) return;
    const float *c = in + (size_t)x * nz + z;
    const ptrdiff_t s = nz;
    out[(size_t)x * nz + z] = 2.0f * RTM_AC0 * c[0]
        + RTM_AC1 * (((c[-s] + c[s]) + c[-1]) + c[1])
        + RTM_AC2 * (((c[-2 * s] + c[2 * s]) + c[-2]) + c[2])
        + RTM_AC3 * (((c[-3 * s] + c[3 * s]) + c[-3]) + c[3])
        + RTM_AC4 * (((c[-4 * s] + c[4 * s]) + c[-4]) + c[4]);
}

template <typename T>
__global__ void k_xcorr(Geom g, const T *src, const T *rcv, double *img, double *slf)
{
    const int z = blockIdx.x * blockDim.x + threadIdx.x;
    const int x = blockIdx.y;
    if (z >= g.nz || x >= g.nx) return;
    const size_t f = (size_t)(x + g.thl) * g.pitch + (z + g.thu);
    const size_t o = (size_t)x * g.pitch + (z + g.thu);
    const double s = (double)src[f], r = (double)rcv[f];
    img[o] += s * r;
    slf[o] += s * s;
}

// ---- launchers ---------------------------------------------------------------------------
size_t step_smem_bytes(int backward, int elem_size, int tx)
{
    return (size_t)(tx + 2 * HALO) * SZ * elem_size * (backward ? 2 : 1);
}

template <typename T, int BWD, int WARPS>
static cudaError_t launch_step_w(const CUtensorMap *tm_u, const CUtensorMap *tm_s,
                                 const StepArgs<T> &a, cudaStream_t s)
{
    const size_t smem = step_smem_bytes(BWD, sizeof(T), StepCfg<T, WARPS>::TXC);
    static bool configured = false;   // attribute set once per instantiation
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(k_step<T, BWD, WARPS>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        configured = true;
    }
    dim3 grid(a.g.tiles_x, a.g.tiles_z);
    k_step<T, BWD, WARPS><<<grid, WARPS * 32, smem, s>>>(*tm_u, *tm_s, a);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_step(int backward, const CUtensorMap *tm_u, const CUtensorMap *tm_s,
                        const StepArgs<T> &a, cudaStream_t s)
{
    const int warps = a.g.tx / StepCfg<T, 4>::RXC;
    if (backward) {
        switch (warps) {
        case 4: return launch_step_w<T, 1, 4>(tm_u, tm_s, a, s);
        case 8: return launch_step_w<T, 1, 8>(tm_u, tm_s, a, s);
        case 16: return launch_step_w<T, 1, 16>(tm_u, tm_s, a, s);
        default: return cudaErrorInvalidValue;
        }
    }
    switch (warps) {
    case 4: return launch_step_w<T, 0, 4>(tm_u, tm_s, a, s);
    case 8: return launch_step_w<T, 0, 8>(tm_u, tm_s, a, s);
    case 16: return launch_step_w<T, 0, 16>(tm_u, tm_s, a, s);
    default: return cudaErrorInvalidValue;
    }
}

template <typename T>
cudaError_t launch_psi(const PsiArgs<T> &a, cudaStream_t s)
{
    const Geom &g = a.g;
    int n = (g.thl - 8) * (g.dimz - 8);
    n = n > (g.thr - 8) * (g.dimz - 8) ? n : (g.thr - 8) * (g.dimz - 8);
    n = n > (g.thu - 8) * (g.dimx - 8) ? n : (g.thu - 8) * (g.dimx - 8);
    n = n > (g.thd - 8) * (g.dimx - 8) ? n : (g.thd - 8) * (g.dimx - 8);
    dim3 grid((n + 255) / 256, 4);
    k_psi<T><<<grid, 256, 0, s>>>(a);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_coef(const Geom &g, const float *vel, int vel_pitch, T *coef, float dx,
                        float dt, cudaStream_t s)
{
    dim3 grid((g.pitch + 127) / 128, g.dimx);
    k_coef<T><<<grid, 128, 0, s>>>(g, vel, vel_pitch, coef, dx, dt);
    return cudaGetLastError();
}

cudaError_t launch_transpose(const float *in, float *out, int rows, int cols, cudaStream_t s)
{
    dim3 grid((cols + 31) / 32, (rows + 31) / 32);
    k_transpose<<<grid, dim3(32, 8), 0, s>>>(in, out, rows, cols);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_image_out(const Geom &g, const double *img, T *out, int accumulate,
                             cudaStream_t s)
{
    dim3 grid((g.nz + 127) / 128, g.nx);
    k_image_out<T><<<grid, 128, 0, s>>>(g, img, out, accumulate);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_field_out(const Geom &g, const T *field, T *out, cudaStream_t s)
{
    dim3 grid((g.dimz + 127) / 128, g.dimx);
    k_field_out<T><<<grid, 128, 0, s>>>(g, field, out);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_field_in(const Geom &g, const T *in, T *field, cudaStream_t s)
{
    dim3 grid((g.pitch + 127) / 128, g.dimx);
    k_field_in<T><<<grid, 128, 0, s>>>(g, in, field);
    return cudaGetLastError();
}

cudaError_t launch_laplacian(int nx, int nz, const float *in, float *out, cudaStream_t s)
{
    dim3 grid((nz + 127) / 128, nx);
    k_laplacian<<<grid, 128, 0, s>>>(nx, nz, in, out);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_xcorr(const Geom &g, const T *src, const T *rcv, double *img, double *slf,
                         cudaStream_t s)
{
    dim3 grid((g.nz + 127) / 128, g.nx);
    k_xcorr<T><<<grid, 128, 0, s>>>(g, src, rcv, img, slf);
    return cudaGetLastError();
}

#define RTM_INSTANTIATE(T)                                                                      \
    template cudaError_t launch_step<T>(int, const CUtensorMap *, const CUtensorMap *,         \
                                        const StepArgs<T> &, cudaStream_t);                    \
    template cudaError_t launch_psi<T>(const PsiArgs<T> &, cudaStream_t);                      \
    template cudaError_t launch_coef<T>(const Geom &, const float *, int, T *, float, float,   \
                                        cudaStream_t);                                         \
    template cudaError_t launch_image_out<T>(const Geom &, const double *, T *, int,           \
                                             cudaStream_t);                                    \
    template cudaError_t launch_field_out<T>(const Geom &, const T *, T *, cudaStream_t);      \
    template cudaError_t launch_field_in<T>(const Geom &, const T *, T *, cudaStream_t);       \
    template cudaError_t launch_xcorr<T>(const Geom &, const T *, const T *, double *,         \
                                         double *, cudaStream_t);
RTM_INSTANTIATE(float)
RTM_INSTANTIATE(double)

}  // namespace rtm
