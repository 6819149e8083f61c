// rtm_kernels.cu -- sm_103a kernels of the RTM engine.
//
//   k_step   one fused time step: 8th-order leapfrog (SRC/stencilDFM.c:7-31), the CPML
//            psi update and corrections (SRC/absorbingBoundaryCondition.c:150-361), source injection
//            (SRC/forward_modeling.c:105-109) or receiver overwrite
//            (SRC/backward_modeling.c:277-281), trace recording, boundary-ring or
//            snapshot storage, reverse-time source reconstruction and the FP64
//            cross-correlation image (SRC/image_conditions.c:20-33).
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

__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
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
// 16-byte asynchronous copy global -> shared (cp.async), its group commit and wait.
__device__ __forceinline__ void cp_async16(void *dst, const void *src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)),
                 "l"(__cvta_generic_to_global(src))
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }
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

// Whether the quad [zq, zq+4) of column x holds a ring cell (a cheap test before ring_index):
// the top and bottom bands span the ring box's columns, the side bands its rows.
__device__ __forceinline__ bool ring_quad(const Geom &g, int x, int zq)
{
    if (x < g.rx0 - 4 || x >= g.rx1 + 4) return false;
    if (x < g.rx0 || x >= g.rx1) return zq < g.rz1 + 4 && zq + 4 > g.rz0 - 4;
    return (zq < g.rz0 && zq + 4 > g.rz0 - 4) || (zq < g.rz1 + 4 && zq + 4 > g.rz1);
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

// ---- CPML psi update of the batched members (k_bpsi) ----------------------------------------
// dpsi of 4 cells from psi along a strided line: rows p[0..3] = f[-4..-1], p[4..7] = f[1..4].
template <typename T>
__device__ __forceinline__ T dpsi_x(const T (&m)[4][4], const T (&p)[4][4], int j)
{
    return (T)RTM_B4 * (p[3][j] - m[0][j]) + (T)RTM_B3 * (p[2][j] - m[1][j])
         + (T)RTM_B2 * (p[1][j] - m[2][j]) + (T)RTM_B1 * (p[0][j] - m[3][j]);
}

// One 4-cell quad of a strip: psi_n = b psi_{n-1} + a D1(u_n) / dx, the reference's loops
// absorbingBoundaryCondition.c:171-189 (left), 219-235 (top), 265-281 (right), 312-328
// (bottom).  strip: 0 left, 1 top, 2 right, 3 bottom; idx: quad index within the strip;
// psi: {left, right, top, bottom}; prof: packed a/b profiles; fresh: psi_{n-1} = 0.
template <typename T>
__device__ __forceinline__ void psi_quad(const Geom &g, T h1, const T *u0, T *const *psi,
                                         const float *const *prof, int strip, int idx, bool fresh)
{
    const size_t P = (size_t)g.pitch;
    if (strip == 0 || strip == 2) {                  // left / right: x-derivative
        const bool left = strip == 0;
        const int th = left ? g.thl : g.thr;
        const int nq = (g.dimz - 8 + 3) / 4;
        if (idx >= (th - 8) * nq) return;
        const int li = 4 + idx / nq, zq = 4 + 4 * (idx % nq);
        const int x = left ? li : g.dimx - g.thr + li;
        T *ps4 = (left ? psi[0] : psi[1]) + (size_t)li * P + zq;
        const T *u = u0 + (size_t)x * P + zq;
        T m[4][4], p[4][4], ps[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            ld4(u - (ptrdiff_t)(4 - k) * (ptrdiff_t)P, m[k]);
            ld4(u + (ptrdiff_t)(k + 1) * (ptrdiff_t)P, p[k]);
        }
        if (fresh) {
#pragma unroll
            for (int j = 0; j < 4; ++j) ps[j] = (T)0;
        } else {
            ld4(ps4, ps);
        }
        const T ab = (T)(left ? prof[0] : prof[2])[li], bb = (T)(left ? prof[1] : prof[3])[li];
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (zq + j < g.dimz - 4) ps[j] = bb * ps[j] + ab * dpsi_x<T>(m, p, j) * h1;
        st4(ps4, ps);
        return;
    }
    int x, zq, zlo, zhi;
    T *ps4;
    const float *pa, *pb;
    if (strip == 1) {                                // top: z-derivative, z in [4, thu-4)
        const int nq = (g.thu - 8 + 3) / 4;
        if (idx >= (g.dimx - 8) * nq) return;
        x = 4 + idx / nq;
        zq = 4 + 4 * (idx % nq);
        zlo = 4; zhi = g.thu - 4;
        ps4 = psi[2] + (size_t)x * g.st + zq;
        pa = prof[4] + zq; pb = prof[5] + zq;
    } else {                                          // bottom: z in [dimz-thd+4, dimz-4)
        zlo = g.dimz - g.thd + 4; zhi = g.dimz - 4;
        const int q0 = zlo & ~3;
        const int nq = (zhi - q0 + 3) / 4;
        if (idx >= (g.dimx - 8) * nq) return;
        x = 4 + idx / nq;
        zq = q0 + 4 * (idx % nq);
        ps4 = psi[3] + (size_t)x * g.sb + (zq - g.zb0);
        pa = prof[6] + (zq - g.zb0); pb = prof[7] + (zq - g.zb0);
    }
    const T *u = u0 + (size_t)x * P + zq;
    T q[12], ps[4];
    {
        T a0[4], a1[4], a2[4];
        ld4(u - 4, a0); ld4(u, a1); ld4(u + 4, a2);
#pragma unroll
        for (int j = 0; j < 4; ++j) { q[j] = a0[j]; q[4 + j] = a1[j]; q[8 + j] = a2[j]; }
    }
    if (fresh) {
#pragma unroll
        for (int j = 0; j < 4; ++j) ps[j] = (T)0;
    } else {
        ld4(ps4, ps);
    }
    const float4 av = *reinterpret_cast<const float4 *>(pa);
    const float4 bv = *reinterpret_cast<const float4 *>(pb);
    const float aa[4] = {av.x, av.y, av.z, av.w}, bb[4] = {bv.x, bv.y, bv.z, bv.w};
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int z = zq + j;
        if (z >= zlo && z < zhi) ps[j] = (T)bb[j] * ps[j] + (T)aa[j] * dpsi_z<T>(q, j) * h1;
    }
    st4(ps4, ps);
}

#include "rtm_march.cuh"
#include "rtm_batch.cuh"

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

// Shot stack on the device (SRC/rtm_iso2d.c:121-126): stack = stack + (float)image, in the
// reference's float arithmetic (the per-shot image rounded to float, then a float sum).  The
// plan's status word is folded into the stack's and cleared, so that a failure of any shot
// surfaces when the stack is read.
__global__ void k_stack_add(Geom g, const double *img, const double *slf, float *acc_img,
                            float *acc_slf, unsigned *plan_status, unsigned *stack_status)
{
    const int z = blockIdx.x * blockDim.x + threadIdx.x;
    const int x = blockIdx.y;
    if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) {
        const unsigned s = *plan_status;
        if (s) {
            atomicOr(stack_status, s);
            *plan_status = 0;
        }
    }
    if (z >= g.nz || x >= g.nx) return;
    const size_t i = (size_t)x * g.nz + z;
    const size_t o = (size_t)x * g.pitch + g.thu + z;
    acc_img[i] = acc_img[i] + (float)img[o];
    acc_slf[i] = acc_slf[i] + (float)slf[o];
}

// The stacked image as the driver writes it: the image stack, or (normalize) the image stack
// divided by the self-image stack (rtm_iso2d.c:150-156, float division), where a pixel with a
// zero self-image stack -- no source energy reached it -- is set to 0 instead of 0/0 or x/0.
__global__ void k_stack_finish(int n, const float *acc_img, const float *acc_slf, int normalize, float *out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float v = acc_img[i];
    if (!normalize) {
        out[i] = v;
        return;
    }
    const float s = acc_slf[i];
    out[i] = s != 0.0f ? v / s : 0.0f;
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
static cudaLaunchAttribute pdl_attr()
{
    cudaLaunchAttribute at;
    at.id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at.val.programmaticStreamSerializationAllowed = 1;
    return at;
}

template <typename T, int BWD, int WARPS>
static cudaError_t configure_step()
{
    static cudaError_t state = cudaErrorNotReady;   // attribute set once per instantiation
    if (state == cudaErrorNotReady) {
        state = cudaFuncSetAttribute(k_step<T, BWD, WARPS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)StepCfg<T, WARPS, BWD>::SMEM);
        // every per-step kernel asks for the same L1/shared split, so alternating kernels do
        // not make the SMs drain and reconfigure the carveout at each launch
        if (state == cudaSuccess)
            state = cudaFuncSetAttribute(k_step<T, BWD, WARPS>,
                                         cudaFuncAttributePreferredSharedMemoryCarveout,
                                         cudaSharedmemCarveoutMaxShared);
    }
    return state;
}

template <typename T, int BWD, int WARPS>
static cudaError_t launch_step_w(const StepMaps &m, const StepArgs<T> &a, int grid, int pdl,
                                 cudaStream_t s)
{
    cudaError_t e = configure_step<T, BWD, WARPS>();
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(WARPS * 32);
    cfg.dynamicSmemBytes = StepCfg<T, WARPS, BWD>::SMEM;
    cfg.stream = s;
    cudaLaunchAttribute at = pdl_attr();
    cfg.attrs = pdl ? &at : nullptr;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, k_step<T, BWD, WARPS>, m, a);
}

template <typename T, int BWD, int WARPS>
static int grid_w(const Geom &g)
{
    static int per_sm = 0, sms = 0;
    if (per_sm == 0) {
        if (configure_step<T, BWD, WARPS>() != cudaSuccess) return 0;
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_step<T, BWD, WARPS>, WARPS * 32,
                                                      StepCfg<T, WARPS, BWD>::SMEM);
        if (per_sm < 1) per_sm = 1;
    }
    const int full = per_sm * sms;
    return g.tiles < full ? g.tiles : full;
}

template <typename T>
int step_grid(int backward, const Geom &g)
{
    const int warps = g.tx / RXC;
    if (backward) {
        if (warps == 4) return grid_w<T, 1, 4>(g);
        if (warps == 8) return grid_w<T, 1, 8>(g);
        if (warps == 16 && sizeof(T) == 4) return grid_w<T, 1, (sizeof(T) == 4 ? 16 : 8)>(g);
        return 0;
    }
    if (warps == 4) return grid_w<T, 0, 4>(g);
    if (warps == 8) return grid_w<T, 0, 8>(g);
    if (warps == 16 && sizeof(T) == 4) return grid_w<T, 0, (sizeof(T) == 4 ? 16 : 8)>(g);
    return 0;
}

size_t step_smem_bytes(int backward, int elem_size, int tx)
{
    const size_t ut8 = (size_t)(tx + 4 * HALO) * SZ, ut = (size_t)(tx + 2 * HALO) * SZ, pt = (size_t)tx * TZ;
    const size_t stage = backward ? ut8 + ut + 3 * pt : ut8 + 2 * pt;
    const size_t ns = (elem_size == 4 && !backward) ? 3 : 2;
    return ns * stage * elem_size;
}

template <typename T>
cudaError_t launch_step(int backward, const StepMaps &maps, const StepArgs<T> &a, int grid,
                        int pdl, cudaStream_t s)
{
    const int warps = a.g.tx / RXC;
    if (grid < 1) return cudaErrorInvalidConfiguration;
    if (backward) {
        if (warps == 4) return launch_step_w<T, 1, 4>(maps, a, grid, pdl, s);
        if (warps == 8) return launch_step_w<T, 1, 8>(maps, a, grid, pdl, s);
        if (warps == 16 && sizeof(T) == 4)
            return launch_step_w<T, 1, (sizeof(T) == 4 ? 16 : 8)>(maps, a, grid, pdl, s);
        return cudaErrorInvalidValue;
    }
    if (warps == 4) return launch_step_w<T, 0, 4>(maps, a, grid, pdl, s);
    if (warps == 8) return launch_step_w<T, 0, 8>(maps, a, grid, pdl, s);
    if (warps == 16 && sizeof(T) == 4)
        return launch_step_w<T, 0, (sizeof(T) == 4 ? 16 : 8)>(maps, a, grid, pdl, s);
    return cudaErrorInvalidValue;
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

cudaError_t launch_stack_add(const Geom &g, const double *img, const double *slf, float *acc_img,
                             float *acc_slf, unsigned *plan_status, unsigned *stack_status, cudaStream_t s)
{
    dim3 grid((g.nz + 127) / 128, g.nx);
    k_stack_add<<<grid, 128, 0, s>>>(g, img, slf, acc_img, acc_slf, plan_status, stack_status);
    return cudaGetLastError();
}

cudaError_t launch_stack_finish(int n, const float *acc_img, const float *acc_slf, int normalize, float *out,
                                cudaStream_t s)
{
    k_stack_finish<<<(n + 255) / 256, 256, 0, s>>>(n, acc_img, acc_slf, normalize, out);
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

void psi_counts_host(const Geom &g, int (&n)[4]) { psi_counts(g, n); }

template <typename T>
cudaError_t launch_bpsi(const BatchIndex *ix, const BMember<T> *mem, const int2 *state, int grid,
                        int pdl, cudaStream_t s)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(256);
    cfg.stream = s;
    cudaLaunchAttribute at = pdl_attr();
    cfg.attrs = pdl ? &at : nullptr;
    cfg.numAttrs = pdl ? 1 : 0;
    static cudaError_t carve = cudaFuncSetAttribute(k_bpsi<T>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                                    cudaSharedmemCarveoutMaxShared);
    if (carve != cudaSuccess) return carve;
    return cudaLaunchKernelEx(&cfg, k_bpsi<T>, ix, mem, state);
}

template <typename T>
cudaError_t launch_bstrip(const BatchIndex *ix, const BMember<T> *mem, int2 *state, unsigned *done, int grid,
                          int pdl, cudaStream_t s)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kStripBlock);
    cfg.stream = s;
    cudaLaunchAttribute at = pdl_attr();
    cfg.attrs = pdl ? &at : nullptr;
    cfg.numAttrs = pdl ? 1 : 0;
    static cudaError_t carve = cudaFuncSetAttribute(k_bstrip<T>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                                    cudaSharedmemCarveoutMaxShared);
    if (carve != cudaSuccess) return carve;
    return cudaLaunchKernelEx(&cfg, k_bstrip<T>, ix, mem, state, done);
}

int strip_items_host(const Geom &g, int ring)
{
    const CorrShape c = corr_shape(g);
    return round_block(c.nA + c.nB) + (ring ? round_block(g.ring_cells) : 0);
}

int strip_blocks_host(const Geom &g)
{
    const CorrShape c = corr_shape(g);
    return round_block(c.nA + c.nB) / kStripBlock;
}

int boundary_tiles_host(const Geom &g) { return boundary_tiles(g); }

template <typename T>
static cudaError_t configure_bstep()
{
    static cudaError_t state = cudaErrorNotReady;
    if (state == cudaErrorNotReady) {
        state = cudaFuncSetAttribute(k_mstep<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)MCfg<T>::SMEM);
        if (state == cudaSuccess)
            state = cudaFuncSetAttribute(k_mstep<T>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                         cudaSharedmemCarveoutMaxShared);
    }
    return state;
}

template <typename T>
int bstep_grid()
{
    static int grid = 0;
    if (grid == 0) {
        if (configure_bstep<T>() != cudaSuccess) return 0;
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mstep<T>, MTHREADS, MCfg<T>::SMEM);
        grid = (per_sm < 1 ? 1 : per_sm) * sms;
    }
    return grid;
}

template <typename T>
cudaError_t launch_bstep(const BatchIndex *ix, const BMember<T> *mem, int2 *state, unsigned *done,
                         int grid, int pdl, cudaStream_t s)
{
    cudaError_t e = configure_bstep<T>();
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(MTHREADS);
    cfg.dynamicSmemBytes = MCfg<T>::SMEM;
    cfg.stream = s;
    cudaLaunchAttribute at = pdl_attr();
    cfg.attrs = pdl ? &at : nullptr;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, k_mstep<T>, ix, mem, state, done);
}

template cudaError_t launch_bpsi<float>(const BatchIndex *, const BMember<float> *, const int2 *, int, int,
                                        cudaStream_t);
template cudaError_t launch_bstep<float>(const BatchIndex *, const BMember<float> *, int2 *, unsigned *,
                                         int, int, cudaStream_t);
template cudaError_t launch_bstrip<float>(const BatchIndex *, const BMember<float> *, int2 *, unsigned *, int,
                                          int, cudaStream_t);
template int bstep_grid<float>();

#define RTM_INSTANTIATE(T)                                                                      \
    template cudaError_t launch_step<T>(int, const StepMaps &, const StepArgs<T> &, int, int,  \
                                        cudaStream_t);                                         \
    template int step_grid<T>(int, const Geom &);                                              \
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
