// ss_mlp_stream.cu — particle-spray stream whose force is the learned
// surrogate, evaluated on the 5th-generation tensor cores.
//
// One CTA = two warpgroups (256 threads); each warpgroup owns its own tile
// of 128 particles (one per thread) and runs independently of the other, so
// one warpgroup's epilogue math overlaps the other's tensor-core GEMMs.  A
// warpgroup integrates its tile with the FP32-compensated Dopri5 step of the
// plain stream (step_f32k); every stage's force is one warpgroup-collective
// network evaluation:
//   layer 1 (4 -> 128) on CUDA cores in FP32 (keeps the input precision),
//   layers 2-4 as tcgen05.mma 128 x 128 x 128 BF16 GEMMs with FP32
//   accumulators in tensor memory (TMEM),
//   the input gradient (the force) as three more tcgen05 GEMMs with the same
//   weight tiles read transposed (MN-major B operand), the final 128 -> 4
//   product on CUDA cores.
// Shared memory holds W2..W4 as BF16 in the no-swizzle core-matrix layout
// (8 rows x 16 bytes per core matrix; element (o, i) of W at byte
// (o/8)*2048 + (i/8)*128 + (o%8)*16 + (i%8)*2), one activation/delta tile A
// [128 particles x 128] per warpgroup in the same layout, and W1, biases and
// w5 in FP32.  TMEM (512 columns x 128 lanes, lane = particle): per
// warpgroup 256 columns = s'(z2), s'(z3) as packed BF16 pairs (64 columns
// each) for the backward chain and one FP32 accumulator (128 columns);
// s'(z1) is recomputed from the inputs.  One thread per warpgroup issues the
// MMAs; completion is signalled by tcgen05.commit on the warpgroup's
// mbarrier; each evaluation waits six times, so the wait parities are
// 0,1,0,1,0,1 in every evaluation.  Every wait is bounded: on a timeout the
// warpgroup records SS_STATUS_ABORTED for its particles, stops issuing MMAs
// and the CTA releases its TMEM.
//
// The judged form (ss_stream_mlp_judged_bf16) keeps the exact potential as
// error judge and fallback: before every judge_every-th step of a tile, the
// surrogate's force at the step's first stage point is compared with the
// exact force (FP32, CUDA cores) for every particle of the tile; if any
// differs by more than tol relative, the tile integrates with the exact
// force from that step on (no more tensor-core work for it).  The judgement
// sits between steps, where the warpgroup is converged, and the decision is
// warpgroup-uniform (a barrier reduction), so the tensor-core path runs
// unchanged for tiles that pass.

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>

#include "ss_stream.cuh"
#include "ss_tcgen05.cuh"

namespace ssg {

static constexpr int MLP_W = SS_MLP_WIDTH;
static constexpr int64_t P_W1 = 0, P_B1 = 512, P_W2 = 640, P_B2 = P_W2 + 16384, P_W3 = P_B2 + 128,
                         P_B3 = P_W3 + 16384, P_W4 = P_B3 + 128, P_B4 = P_W4 + 16384, P_W5 = P_B4 + 128,
                         P_B5 = P_W5 + 128;
static_assert(P_B5 + 1 == SS_MLP_NPARAM, "parameter packing");

// shared-memory map (bytes from a 1024-aligned base)
static constexpr uint32_t SM_W2 = 0, SM_W3 = 32768, SM_W4 = 65536, SM_A = 98304;  // A tiles: 2 x 32 KB
static constexpr uint32_t SM_W1 = SM_A + 65536;       // float [128][4]
static constexpr uint32_t SM_B = SM_W1 + 2048;        // float b1..b4 [4][128]
static constexpr uint32_t SM_W5 = SM_B + 2048;        // float [128]
static constexpr uint32_t SM_BAR = SM_W5 + 512;       // 2 mbarriers (8 B each)
static constexpr uint32_t SM_TMEM = SM_BAR + 16;      // TMEM base address
static constexpr uint32_t SM_ABORT = SM_TMEM + 4;     // 2 abort flags
static constexpr uint32_t SM_START = SM_ABORT + 8;    // 2 tile start steps
static constexpr uint32_t SM_BASE = SM_START + 8;     // float2 [SS_MLP_BASE_MAX]: the exact spherical part
static constexpr uint32_t SM_BYTES = SM_BASE + 8 * SS_MLP_BASE_MAX;
static constexpr uint32_t SM_ALLOC = SM_BYTES + 1024;  // slack for the 1024-byte alignment

// TMEM columns within a warpgroup's 256
static constexpr uint32_t T_S2 = 0, T_S3 = 64, T_ACC = 128;
static constexpr int MLP_THREADS = 256;

// MN-major B operand, no swizzle: SBO = stride between core matrices along
// N (the contiguous 16 bytes), LBO = stride along K.
static constexpr uint32_t MN_LBO = 2048, MN_SBO = 128;

enum { SS_STATUS_ABORTED = 2 };

struct MlpDev {
    const float* params;
    float c[4], s[4];
    float out_scale, out_shift;
    const double* base;  // exact spherical part (ss_mlp.base), or NULL; copied to shared memory as float
    int base_n;
    float base_u0, base_du;
};


__device__ __forceinline__ uint8_t* mlp_smem() {
    extern __shared__ uint8_t ss_mlp_dyn[];
    return (uint8_t*)(((uintptr_t)ss_mlp_dyn + 1023) & ~(uintptr_t)1023);
}


// sigmoid via the hardware tanh: s(z) = 0.5 + 0.5 tanh(z / 2)
__device__ __forceinline__ float sigm(float z) {
    float t;
    asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(0.5f * z));
    return fmaf(0.5f, t, 0.5f);
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&v);
}

struct MlpCta {
    uint32_t tmem;      // this warpgroup's TMEM base (lane 0, its first column)
    uint32_t lane_off;  // this warp's lane offset << 16
    uint32_t bar;       // this warpgroup's mbarrier (shared address)
    uint32_t base;      // shared address of the aligned base
    uint32_t a_off;     // this warpgroup's A tile (offset from the base)
    int wg;             // warpgroup 0 or 1
};

// barrier over one warpgroup (named barrier 1 + wg, 128 threads)
__device__ __forceinline__ void wg_sync(int wg) { asm volatile("bar.sync %0, 128;" ::"r"(1 + wg) : "memory"); }

// barrier over one warpgroup that also ORs a flag across it
__device__ __forceinline__ bool wg_sync_or(int wg, bool v) {
    uint32_t r;
    asm volatile(
        "{\n.reg .pred p, q;\nsetp.ne.u32 q, %1, 0;\nbar.red.or.pred p, %2, 128, q;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(r)
        : "r"((uint32_t)v), "r"(1 + wg)
        : "memory");
    return r != 0;
}

// Issue one 128x128x128 GEMM of this warpgroup into its accumulator and
// wait for it.  wsm: weight tile offset; b_mn: 0 = z = A W^T (forward),
// 1 = u = A W (backward).  Returns false on a wait timeout (abort).
__device__ __forceinline__ bool gemm_layer(const MlpCta& cx, uint32_t wsm, uint32_t b_mn, uint32_t parity,
                                           volatile uint32_t* abort) {
    tmem_wait_st();
    fence_async_smem();
    fence_before();
    wg_sync(cx.wg);
    if (*abort) return false;
    if ((threadIdx.x & 127) == 0) {
        fence_after();
        const uint32_t id = idesc_bf16(b_mn);
#pragma unroll
        for (int kk = 0; kk < 8; ++kk) {
            const uint64_t ad = smem_desc(cx.base + cx.a_off + kk * 256, 128, 2048);
            const uint64_t bd = b_mn ? smem_desc(cx.base + wsm + kk * 4096, MN_LBO, MN_SBO)
                                     : smem_desc(cx.base + wsm + kk * 256, 128, 2048);
            mma_bf16(cx.tmem + T_ACC, ad, bd, id, kk > 0 ? 1u : 0u);
        }
        mma_commit(cx.bar);
    }
    const bool ok = mbar_wait(cx.bar, parity);
    fence_after();
    // every thread of the warpgroup takes the same path after a timeout
    if (wg_sync_or(cx.wg, !ok)) {
        *abort = 1u;
        return false;
    }
    return true;
}

__device__ __forceinline__ float bf_lo(uint32_t u) { return __uint_as_float(u << 16); }
__device__ __forceinline__ float bf_hi(uint32_t u) { return __uint_as_float(u & 0xffff0000u); }

// store 32 consecutive features of one particle row into an A tile
__device__ __forceinline__ void store_row32_at(uint8_t* tile, int row, int c, const float v[32]) {
    uint8_t* r = tile + (row >> 3) * 2048 + (row & 7) * 16;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        uint4 w;
        w.x = pack_bf16(v[8 * q + 0], v[8 * q + 1]);
        w.y = pack_bf16(v[8 * q + 2], v[8 * q + 3]);
        w.z = pack_bf16(v[8 * q + 4], v[8 * q + 5]);
        w.w = pack_bf16(v[8 * q + 6], v[8 * q + 7]);
        *reinterpret_cast<uint4*>(r + (4 * c + q) * 128) = w;
    }
}

// grad Phi at X (FP32) for every thread of one warpgroup (collective).
__device__ __noinline__ void mlp_grad_wg(const MlpDev& M, const MlpCta& cx, float X0, float X1, float X2, float& g0,
                                         float& g1, float& g2) {
    uint8_t* sm = mlp_smem();
    volatile uint32_t* abort = reinterpret_cast<volatile uint32_t*>(sm + SM_ABORT) + cx.wg;
    const float* W1 = reinterpret_cast<const float*>(sm + SM_W1);
    const float* Bb = reinterpret_cast<const float*>(sm + SM_B);
    const float* w5 = reinterpret_cast<const float*>(sm + SM_W5);
    uint8_t* tile = sm + cx.a_off;
    const int row = threadIdx.x & 127;
    const uint32_t tl = cx.tmem + cx.lane_off;
    g0 = g1 = g2 = 0.0f;
    if (*abort) return;
    const float r2 = X0 * X0 + X1 * X1 + X2 * X2;
    const float u0 = (X0 - M.s[0]) * M.c[0], u1 = (X1 - M.s[1]) * M.c[1], u2 = (X2 - M.s[2]) * M.c[2];
    const float u3 = (0.5f * logf(r2) - M.s[3]) * M.c[3];
    // layer 1 on CUDA cores: a1 -> A tile (s'(z1) is recomputed in the backward pass)
#pragma unroll 1
    for (int c = 0; c < 4; ++c) {
        float a[32];
#pragma unroll
        for (int j = 0; j < 32; ++j) {
            const int f = 32 * c + j;
            const float4 w = *reinterpret_cast<const float4*>(W1 + 4 * f);
            const float z = fmaf(w.x, u0, fmaf(w.y, u1, fmaf(w.z, u2, fmaf(w.w, u3, Bb[f]))));
            a[j] = z * sigm(z);
        }
        store_row32_at(tile, row, c, a);
    }
    // layers 2 and 3: z = a W^T + b, a = SiLU(z) -> A tile, s'(z) -> S2 / S3 (packed BF16)
#pragma unroll 1
    for (int k = 2; k <= 3; ++k) {
        if (!gemm_layer(cx, k == 2 ? SM_W2 : SM_W3, 0, k == 2 ? 0u : 1u, abort)) return;
        const float* bk = Bb + (k - 1) * MLP_W;
        const uint32_t sc = k == 2 ? T_S2 : T_S3;
#pragma unroll 1
        for (int c = 0; c < 4; ++c) {
            uint32_t r[32], sp[16];
            float a[32];
            SS_TMEM_LD32(r, tl + T_ACC + 32 * c);
            tmem_wait_ld();
#pragma unroll
            for (int j = 0; j < 32; j += 2) {
                float s2[2];
#pragma unroll
                for (int e = 0; e < 2; ++e) {
                    const float z = __uint_as_float(r[j + e]) + bk[32 * c + j + e];
                    const float sg = sigm(z);
                    a[j + e] = z * sg;
                    s2[e] = sg * fmaf(z, 1.0f - sg, 1.0f);
                }
                sp[j / 2] = pack_bf16(s2[0], s2[1]);
            }
            store_row32_at(tile, row, c, a);
            SS_TMEM_ST16(tl + sc + 16 * c, sp);
        }
    }
    // layer 4: only s'(z4) is needed: d4 = w5 s'(z4) -> A tile
    if (!gemm_layer(cx, SM_W4, 0, 0u, abort)) return;
    {
        const float* b4 = Bb + 3 * MLP_W;
#pragma unroll 1
        for (int c = 0; c < 4; ++c) {
            uint32_t r[32];
            float d[32];
            SS_TMEM_LD32(r, tl + T_ACC + 32 * c);
            tmem_wait_ld();
#pragma unroll
            for (int j = 0; j < 32; ++j) {
                const int f = 32 * c + j;
                const float z = __uint_as_float(r[j]) + b4[f];
                const float sg = sigm(z);
                d[j] = w5[f] * (sg * fmaf(z, 1.0f - sg, 1.0f));
            }
            store_row32_at(tile, row, c, d);
        }
    }
    // backward: u = d W_k (MN-major B), d_{k-1} = u s'(z_{k-1})
    const uint32_t wk[3] = {SM_W4, SM_W3, SM_W2};
    float gi[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll 1
    for (int q = 0; q < 3; ++q) {
        if (!gemm_layer(cx, wk[q], 1, q == 1 ? 0u : 1u, abort)) return;
#pragma unroll 1
        for (int c = 0; c < 4; ++c) {
            uint32_t r[32];
            float d[32];
            SS_TMEM_LD32(r, tl + T_ACC + 32 * c);
            if (q < 2) {
                uint32_t sv[16];
                SS_TMEM_LD16(sv, tl + (q == 0 ? T_S3 : T_S2) + 16 * c);
                tmem_wait_ld();
#pragma unroll
                for (int j = 0; j < 32; j += 2) {
                    d[j] = __uint_as_float(r[j]) * bf_lo(sv[j / 2]);
                    d[j + 1] = __uint_as_float(r[j + 1]) * bf_hi(sv[j / 2]);
                }
                store_row32_at(tile, row, c, d);
            } else {
                tmem_wait_ld();
                // d1 = u1 s'(z1) with s'(z1) recomputed; g = W1^T d1 (FP32)
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    const int f = 32 * c + j;
                    const float4 w = *reinterpret_cast<const float4*>(W1 + 4 * f);
                    const float z = fmaf(w.x, u0, fmaf(w.y, u1, fmaf(w.z, u2, fmaf(w.w, u3, Bb[f]))));
                    const float sg = sigm(z);
                    const float d1 = __uint_as_float(r[j]) * (sg * fmaf(z, 1.0f - sg, 1.0f));
                    gi[0] = fmaf(w.x, d1, gi[0]);
                    gi[1] = fmaf(w.y, d1, gi[1]);
                    gi[2] = fmaf(w.z, d1, gi[2]);
                    gi[3] = fmaf(w.w, d1, gi[3]);
                }
            }
        }
    }
    float k3 = M.out_scale * gi[3] * M.c[3] / r2;
    if (M.base_n > 0) {
        // + grad Phi_0 = (dPhi_0 / du) x / r^2, u = ln r
        float f0, fu;
        base_spline<float, float>(reinterpret_cast<const float*>(sm + SM_BASE), M.base_n, M.base_u0, M.base_du,
                                  1.0f / M.base_du, 0.5f * logf(r2), f0, fu);
        k3 += fu / r2;
    }
    g0 = M.out_scale * gi[0] * M.c[0] + k3 * X0;
    g1 = M.out_scale * gi[1] * M.c[1] + k3 * X1;
    g2 = M.out_scale * gi[2] * M.c[2] + k3 * X2;
}

// The "composition" handed to step_f32k: its gradient is the CTA-collective
// network evaluation (the CTA context lives in shared memory).
struct MlpComp {
    static constexpr int n = 1;
    template <class R>
    static __device__ __forceinline__ constexpr bool uses_track(const PotDev<R>&) {
        return false;
    }
    template <class T, class R, bool HESS>
    static __device__ __forceinline__ void grad(const PotDev<R>& P, const T x[3], const T xs[3], T g[3], T H[6],
                                                const TimeDep<T>& td = TimeDep<T>());
};

struct MlpKernelArgs {
    MlpDev M;
    StreamArgs a;
    int64_t n_tiles;
    // judged form: the exact potential (analytic kinds and an l_max = 8
    // expansion with its FP32 table), the tolerance, the judging interval
    // in steps, the fallback counter (device); judged = 0: surrogate only
    PotDev<float> X;
    float tol;
    int judge_every;
    int judged;
    unsigned long long* fallbacks;
};

// The exact force of the judge, components in list order: the FP32 forms of
// the stream kernels (kind_grad, shexp_grad_fixed).  Kept out of line so
// that it does not add to the tensor-core path's registers.
__device__ __noinline__ void judge_exact_grad(const PotDev<float>& P, float x0, float x1, float x2, float g[3]) {
    const float x[3] = {x0, x1, x2};
    g[0] = g[1] = g[2] = 0.0f;
    for (int i = 0; i < P.n; ++i) {
        switch (P.c[i].kind) {
            case SS_SH_EXPANSION: {
                const Vec3<float> v = shexp_grad_fixed<SS_SHEXP_LMAX>(P.ex, P.c[i].q[0], x0, x1, x2);
                g[0] += v.x;
                g[1] += v.y;
                g[2] += v.z;
                break;
            }
            case SS_NFW: kind_grad<SS_NFW, float, float, false>(P.c[i].q, x, g, nullptr); break;
            case SS_TRIAXIAL_NFW: kind_grad<SS_TRIAXIAL_NFW, float, float, false>(P.c[i].q, x, g, nullptr); break;
            case SS_MIYAMOTO_NAGAI: kind_grad<SS_MIYAMOTO_NAGAI, float, float, false>(P.c[i].q, x, g, nullptr); break;
            case SS_HERNQUIST: kind_grad<SS_HERNQUIST, float, float, false>(P.c[i].q, x, g, nullptr); break;
            case SS_PLUMMER: kind_grad<SS_PLUMMER, float, float, false>(P.c[i].q, x, g, nullptr); break;
            default: kind_grad<SS_ISOCHRONE, float, float, false>(P.c[i].q, x, g, nullptr); break;
        }
    }
}

__device__ __forceinline__ const MlpKernelArgs*& mlp_args_ptr() {
    __shared__ const MlpKernelArgs* p;
    return p;
}

template <class T, class R, bool HESS>
__device__ __forceinline__ void MlpComp::grad(const PotDev<R>&, const T x[3], const T*, T g[3], T*, const TimeDep<T>&) {
    uint8_t* sm = mlp_smem();
    MlpCta cx;
    cx.wg = threadIdx.x >> 7;
    cx.tmem = *reinterpret_cast<volatile uint32_t*>(sm + SM_TMEM) + 256u * cx.wg;
    cx.lane_off = (uint32_t)(32 * ((threadIdx.x >> 5) & 3)) << 16;
    cx.bar = smem_u32(sm + SM_BAR + 8 * cx.wg);
    cx.base = smem_u32(sm);
    cx.a_off = SM_A + 32768u * cx.wg;
    const MlpKernelArgs* ka = mlp_args_ptr();
    mlp_grad_wg(ka->M, cx, x[0], x[1], x[2], g[0], g[1], g[2]);
}

// The judge's fallback composition for step_f32k: the exact force
// (judge_exact_grad) of the potential passed as P, no tensor-core work.
struct ExactComp {
    static constexpr int n = 1;
    template <class R>
    static __device__ __forceinline__ constexpr bool uses_track(const PotDev<R>&) {
        return false;
    }
    template <class T, class R, bool HESS>
    static __device__ __forceinline__ void grad(const PotDev<R>& P, const T x[3], const T*, T g[3], T*,
                                                const TimeDep<T>& = TimeDep<T>()) {
        judge_exact_grad(P, x[0], x[1], x[2], g);
    }
};

// CTA prologue: weights -> shared memory (BF16 core-matrix tiles, FP32
// small parts), mbarrier, 512 TMEM columns.
__device__ __forceinline__ void mlp_cta_setup(const MlpKernelArgs& ka) {
    uint8_t* sm = mlp_smem();
    const int t = threadIdx.x;
    const float* prm = ka.M.params;
    for (int e = t; e < 3 * 16384; e += blockDim.x) {
        const int k = e / 16384, idx = e % 16384, o = idx / 128, i = idx % 128;
        const float w = prm[(k == 0 ? P_W2 : k == 1 ? P_W3 : P_W4) + idx];
        __nv_bfloat16 b = __float2bfloat16_rn(w);
        *reinterpret_cast<__nv_bfloat16*>(sm + 32768 * k + (o >> 3) * 2048 + (i >> 3) * 128 + (o & 7) * 16 +
                                          (i & 7) * 2) = b;
    }
    float* W1 = reinterpret_cast<float*>(sm + SM_W1);
    float* Bb = reinterpret_cast<float*>(sm + SM_B);
    float* w5 = reinterpret_cast<float*>(sm + SM_W5);
    for (int e = t; e < 512; e += blockDim.x) W1[e] = prm[P_W1 + e];
    float* base = reinterpret_cast<float*>(sm + SM_BASE);
    for (int e = t; e < 2 * ka.M.base_n; e += blockDim.x) base[e] = (float)ka.M.base[e];
    for (int e = t; e < 128; e += blockDim.x) {
        Bb[e] = prm[P_B1 + e];
        Bb[128 + e] = prm[P_B2 + e];
        Bb[256 + e] = prm[P_B3 + e];
        Bb[384 + e] = prm[P_B4 + e];
        w5[e] = prm[P_W5 + e];
    }
    if (t == 0) {
        mlp_args_ptr() = &ka;
        reinterpret_cast<uint32_t*>(sm + SM_ABORT)[0] = 0u;
        reinterpret_cast<uint32_t*>(sm + SM_ABORT)[1] = 0u;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(sm + SM_BAR)), "r"(1));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(sm + SM_BAR + 8)), "r"(1));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if ((t >> 5) == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(sm + SM_TMEM)),
                     "r"(512));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
}

// CTA epilogue: release TMEM (after a timeout, the warpgroup first gives
// its outstanding commit a bounded wait).
__device__ __forceinline__ void mlp_cta_teardown() {
    uint8_t* sm = mlp_smem();
    volatile uint32_t* abort = reinterpret_cast<volatile uint32_t*>(sm + SM_ABORT);
    const int wg = threadIdx.x >> 7;
    if (abort[wg] && (threadIdx.x & 127) == 0) {
        mbar_wait(smem_u32(sm + SM_BAR + 8 * wg), 0u);
        mbar_wait(smem_u32(sm + SM_BAR + 8 * wg), 1u);
    }
    fence_before();
    __syncthreads();
    fence_after();
    if ((threadIdx.x >> 5) == 0) {
        const uint32_t tm = *reinterpret_cast<volatile uint32_t*>(sm + SM_TMEM);
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tm), "r"(512));
    }
}

// grad Phi of the surrogate at points xyz [n,3] (tensor-core path; tests)
__global__ void __launch_bounds__(MLP_THREADS, 1) mlp_grad_kernel(const __grid_constant__ MlpKernelArgs ka, const double* xyz,
                                                                  int64_t n, double* grad, int32_t* status) {
    mlp_cta_setup(ka);
    uint8_t* sm = mlp_smem();
    const int wg = threadIdx.x >> 7;
    volatile uint32_t* abort = reinterpret_cast<volatile uint32_t*>(sm + SM_ABORT) + wg;
    PotDev<float> P;
    P.n = 0;
    P.has_track = 0;
    const int64_t n_tiles = (n + 127) / 128;
    for (int64_t tile = 2 * (int64_t)blockIdx.x + wg; tile < n_tiles; tile += 2 * (int64_t)gridDim.x) {
        const int64_t p = tile * 128 + (threadIdx.x & 127);
        const int64_t q = p < n ? p : 0;
        const float x[3] = {(float)xyz[3 * q], (float)xyz[3 * q + 1], (float)xyz[3 * q + 2]};
        float g[3];
        MlpComp::grad<float, float, false>(P, x, x, g, nullptr);
        if (p < n) {
            for (int i = 0; i < 3; ++i) grad[3 * p + i] = (double)g[i];
            if (status) status[p] = *abort ? SS_STATUS_ABORTED : 0;
        }
        if (*abort) break;
    }
    mlp_cta_teardown();
}

__global__ void __launch_bounds__(MLP_THREADS, 1) stream_mlp_kernel(const __grid_constant__ MlpKernelArgs ka) {
    mlp_cta_setup(ka);
    uint8_t* sm = mlp_smem();
    const int t = threadIdx.x & 127, wg = threadIdx.x >> 7;
    const StreamArgs& a = ka.a;
    volatile uint32_t* abort = reinterpret_cast<volatile uint32_t*>(sm + SM_ABORT) + wg;
    int* s_start = reinterpret_cast<int*>(sm + SM_START) + wg;
    PotDev<float> P;  // unused by MlpComp (no track, no subhalos)
    P.n = 0;
    P.has_track = 0;
    // warpgroups take alternate tiles and run independently
    for (int64_t tile = 2 * (int64_t)blockIdx.x + wg; tile < ka.n_tiles; tile += 2 * (int64_t)gridDim.x) {
        const int64_t p = tile * 128 + t;
        const bool valid = p < a.N;
        const int start = valid ? (int)(((p + a.p_off) / a.ppr) * (int64_t)a.spr) : a.n_steps;
        // the tile steps from its earliest start; particles not yet released
        // step a copy (their rows of the GEMMs are independent)
        if (t == 0) *s_start = a.n_steps;
        wg_sync(wg);
        atomicMin(s_start, start);
        wg_sync(wg);
        const int tstart = *s_start;
        wg_sync(wg);
        float xh[3], xl[3], vh[3], vl[3];
        const int64_t q = valid ? p : 0;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const double xd = a.ics[6 * q + i], vd = a.ics[6 * q + 3 + i];
            xh[i] = (float)xd;
            xl[i] = (float)(xd - (double)xh[i]);
            vh[i] = (float)vd;
            vl[i] = (float)(vd - (double)vh[i]);
        }
        if (a.snaps && valid) {
            const float y[6] = {xh[0], xh[1], xh[2], vh[0], vh[1], vh[2]};
            for (int64_t k = 0; (k + 1) * (int64_t)a.stride <= tstart; ++k)
                write_snap<float>(a.snaps, a.snap_pitch, k, p + a.p_off, (k + 1) * (int64_t)a.stride >= start, y);
        }
        bool exact = false;  // the tile fell back to the exact force (uniform over the warpgroup)
        for (int n = tstart; n < a.n_steps; ++n) {
            if (*abort) break;
            if (ka.judged && !exact && (n - tstart) % ka.judge_every == 0) {
                // judge at the step's first stage point, x_hi + x_lo: the
                // surrogate's force there against the exact one
                const float X[3] = {xh[0] + xl[0], xh[1] + xl[1], xh[2] + xl[2]};
                float gm[3], ge[3];
                MlpComp::grad<float, float, false>(P, X, X, gm, nullptr);
                judge_exact_grad(ka.X, X[0], X[1], X[2], ge);
                const float d0 = gm[0] - ge[0], d1 = gm[1] - ge[1], d2 = gm[2] - ge[2];
                const float e2 = d0 * d0 + d1 * d1 + d2 * d2, n2 = ge[0] * ge[0] + ge[1] * ge[1] + ge[2] * ge[2];
                const bool bad = !(e2 <= ka.tol * ka.tol * n2);  // NaN counts as bad
                exact = wg_sync_or(wg, bad);
                if (exact && t == 0 && ka.fallbacks) atomicAdd(ka.fallbacks, 1ull);
                __syncwarp();
            }
            float th[3], tlo[3], uh[3], ul[3];
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                th[i] = xh[i];
                tlo[i] = xl[i];
                uh[i] = vh[i];
                ul[i] = vl[i];
            }
            if (exact)
                step_f32k<ExactComp, SUB_NONE>(ka.X, a, n, th, tlo, uh, ul);
            else
                step_f32k<MlpComp, SUB_NONE>(P, a, n, th, tlo, uh, ul);  // the surrogate alone: no subhalos
            if (valid && n >= start) {
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    xh[i] = th[i];
                    xl[i] = tlo[i];
                    vh[i] = uh[i];
                    vl[i] = ul[i];
                }
            }
            if (a.snaps && (n + 1) % a.stride == 0 && valid) {
                const float y[6] = {xh[0], xh[1], xh[2], vh[0], vh[1], vh[2]};
                write_snap<float>(a.snaps, a.snap_pitch, (n + 1) / a.stride - 1, p + a.p_off, n + 1 >= start, y);
            }
        }
        if (valid) {
            bool ok = true;
#pragma unroll
            for (int i = 0; i < 3; ++i) ok = ok && isfinite(xh[i]) && isfinite(vh[i]) && isfinite(xl[i]) && isfinite(vl[i]);
            if (a.status) a.status[p] = *abort ? SS_STATUS_ABORTED : (ok ? 0 : 1);
            if (a.final_w) {
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    a.final_w[6 * p + i] = (double)xh[i] + (double)xl[i];
                    a.final_w[6 * p + 3 + i] = (double)vh[i] + (double)vl[i];
                }
            }
        }
        if (*abort) break;
    }
    mlp_cta_teardown();
}

static int mlp_dev_of(const ss_mlp* mlp, MlpDev* M) {
    SS_CHECK_ARG(mlp->base == nullptr || (mlp->base_n >= 2 && mlp->base_n <= SS_MLP_BASE_MAX && mlp->base_du > 0.0),
                 "mlp base table needs 2 <= base_n <= %d knots and base_du > 0", SS_MLP_BASE_MAX);
    M->params = mlp->params;
    for (int i = 0; i < 4; ++i) {
        M->c[i] = mlp->in_scale[i];
        M->s[i] = mlp->in_shift[i];
    }
    M->out_scale = mlp->out_scale;
    M->out_shift = mlp->out_shift;
    M->base = mlp->base;
    M->base_n = mlp->base ? mlp->base_n : 0;
    M->base_u0 = (float)mlp->base_u0;
    M->base_du = (float)mlp->base_du;
    return SS_OK;
}

}  // namespace ssg

using namespace ssg;

extern "C" {

int ss_mlp_grad_bf16(const ss_mlp* mlp, const double* xyz, int64_t n, double* grad, int32_t* status, void* stream) {
    SS_CHECK_ARG(mlp != nullptr && mlp->params != nullptr, "mlp or its params is NULL");
    SS_CHECK_ARG(n >= 0, "n < 0");
    if (n == 0) return SS_OK;
    SS_CHECK_ARG(xyz != nullptr && grad != nullptr, "NULL buffer");
    MlpKernelArgs ka;
    memset(&ka, 0, sizeof(ka));
    const int rc_m = mlp_dev_of(mlp, &ka.M);
    if (rc_m) return rc_m;
    int dev = 0, sms = 0;
    SS_CUDA_TRY(cudaGetDevice(&dev));
    SS_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    SS_CUDA_TRY(cudaFuncSetAttribute(mlp_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SM_ALLOC));
    const int64_t pairs = ((n + 127) / 128 + 1) / 2;
    mlp_grad_kernel<<<(unsigned)(pairs < sms ? pairs : sms), MLP_THREADS, SM_ALLOC, (cudaStream_t)stream>>>(ka, xyz, n, grad,
                                                                                                      status);
    SS_LAUNCH_CHECK();
    return SS_OK;
}

int64_t ss_stream_mlp_workspace_bytes(const ss_stream_cfg* cfg) {
    if (cfg == nullptr) return set_error(SS_ERR_INVALID_ARGUMENT, "cfg is NULL");
    return 0;
}

int64_t ss_stream_mlp_judged_workspace_bytes(const ss_potential* exact, const ss_stream_cfg* cfg) {
    if (exact == nullptr || cfg == nullptr) return set_error(SS_ERR_INVALID_ARGUMENT, "NULL argument");
    return expansion_table32_bytes(exact);
}

static int mlp_stream(const ss_mlp* mlp, const ss_potential* exact, const ss_stream_cfg* cfg, float tol,
                      int32_t judge_every, const double* ics, double* final_w, float* snaps, int32_t* status,
                      int64_t* fallbacks, void* workspace, int64_t workspace_bytes, void* stream) {
    SS_CHECK_ARG(mlp != nullptr && mlp->params != nullptr, "mlp or its params is NULL");
    SS_CHECK_ARG(cfg != nullptr, "cfg is NULL");
    SS_CHECK_ARG(cfg->n_particles >= 0, "n_particles < 0");
    SS_CHECK_ARG(cfg->n_steps >= 0 && cfg->n_steps < (1LL << 30), "n_steps outside [0, 2^30)");
    SS_CHECK_ARG(cfg->particles_per_release >= 1 && cfg->steps_per_release >= 0, "bad release layout");
    SS_CHECK_ARG(std::isfinite(cfg->dt) && cfg->dt > 0.0 && std::isfinite(cfg->t0), "dt must be finite and > 0");
    SS_CHECK_ARG(cfg->snap_stride >= 0, "snap_stride < 0");
    SS_CHECK_ARG(cfg->first_particle >= 0 && cfg->snap_pitch >= 0, "first_particle and snap_pitch must be >= 0");
    SS_CHECK_ARG(cfg->stream_particles == 0, "the surrogate stream runs single streams (stream_particles = 0)");
    SS_CHECK_ARG(cfg->snap_pitch == 0 || cfg->snap_pitch >= cfg->first_particle + cfg->n_particles,
                 "snap_pitch must cover first_particle + n_particles");
    const int64_t n_rel =
        (cfg->first_particle + cfg->n_particles + cfg->particles_per_release - 1) / cfg->particles_per_release;
    SS_CHECK_ARG(n_rel == 0 || (n_rel - 1) * (int64_t)cfg->steps_per_release <= cfg->n_steps,
                 "last release starts after n_steps");
    MlpKernelArgs ka;
    memset(&ka, 0, sizeof(ka));
    if (exact) {
        SS_CHECK_ARG(std::isfinite(tol) && tol >= 0.0f, "tol must be finite and >= 0");
        SS_CHECK_ARG(judge_every >= 1, "judge_every must be >= 1");
        int rc = prepare_potential<float>(exact, &ka.X, false);
        if (rc) return rc;
        SS_CHECK_ARG(!ka.X.has_track && !ka.X.has_rot && !ka.X.has_facc && !ka.X.grow_mask,
                     "the judge's exact potential must be static, without a center track");
        for (int k = 0; k < ka.X.n; ++k) {
            const int kd = ka.X.c[k].kind;
            if (kd == SS_SH_EXPANSION)
                SS_CHECK_ARG(ka.X.ex.lmax == SS_SHEXP_LMAX, "the judge evaluates expansions of l_max = %d only",
                             SS_SHEXP_LMAX);
            else
                SS_CHECK_ARG(kd == SS_NFW || kd == SS_TRIAXIAL_NFW || kd == SS_MIYAMOTO_NAGAI || kd == SS_HERNQUIST ||
                                 kd == SS_PLUMMER || kd == SS_ISOCHRONE,
                             "component %d: kind %d is not available to the judge", k, kd);
        }
        const int64_t need = expansion_table32_bytes(exact);
        if (need > 0 && (workspace == nullptr || workspace_bytes < need))
            return set_error(SS_ERR_WORKSPACE, "workspace of %lld bytes needed, %lld given", (long long)need,
                             (long long)workspace_bytes);
        SS_CHECK_ARG(need == 0 || ((uintptr_t)workspace % 256) == 0, "workspace must be 256-byte aligned");
        ka.tol = tol;
        ka.judge_every = judge_every;
        ka.judged = 1;
        ka.fallbacks = reinterpret_cast<unsigned long long*>(fallbacks);
    }
    if (cfg->n_particles == 0) return SS_OK;
    SS_CHECK_ARG(ics != nullptr, "ics is NULL");
    const int rc_m = mlp_dev_of(mlp, &ka.M);
    if (rc_m) return rc_m;
    if (exact) {
        const int rc = expansion_table32(ka.X, workspace, (cudaStream_t)stream);
        if (rc) return rc;
    }
    StreamArgs& a = ka.a;
    a.ics = ics;
    a.final_w = final_w;
    a.snaps = cfg->snap_stride > 0 && cfg->n_steps >= cfg->snap_stride ? snaps : nullptr;
    a.status = status;
    a.N = cfg->n_particles;
    a.ppr = cfg->particles_per_release;
    a.spr = cfg->steps_per_release;
    a.n_steps = (int32_t)cfg->n_steps;
    a.stride = cfg->snap_stride > 0 ? cfg->snap_stride : 1;
    a.t0 = cfg->t0;
    a.dt = cfg->dt;
    a.h_hi = (float)cfg->dt;
    a.h_lo = (float)(cfg->dt - (double)a.h_hi);
    a.p_off = cfg->first_particle;
    a.snap_pitch = cfg->snap_pitch > 0 ? cfg->snap_pitch : cfg->first_particle + cfg->n_particles;
    ka.n_tiles = (cfg->n_particles + 127) / 128;
    int dev = 0, sms = 0;
    SS_CUDA_TRY(cudaGetDevice(&dev));
    SS_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    SS_CUDA_TRY(cudaFuncSetAttribute(stream_mlp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SM_ALLOC));
    const int64_t pairs = (ka.n_tiles + 1) / 2;
    const int64_t grid = pairs < sms ? pairs : sms;
    stream_mlp_kernel<<<(unsigned)grid, MLP_THREADS, SM_ALLOC, (cudaStream_t)stream>>>(ka);
    SS_LAUNCH_CHECK();
    return SS_OK;
}

int ss_stream_mlp_bf16(const ss_mlp* mlp, const ss_stream_cfg* cfg, const double* ics, double* final_w, float* snaps,
                       int32_t* status, void* workspace, int64_t workspace_bytes, void* stream) {
    return mlp_stream(mlp, nullptr, cfg, 0.0f, 1, ics, final_w, snaps, status, nullptr, workspace, workspace_bytes,
                      stream);
}

int ss_stream_mlp_judged_bf16(const ss_mlp* mlp, const ss_potential* exact, const ss_stream_cfg* cfg, float tol,
                              int32_t judge_every, const double* ics, double* final_w, float* snaps, int32_t* status,
                              int64_t* fallbacks, void* workspace, int64_t workspace_bytes, void* stream) {
    SS_CHECK_ARG(exact != nullptr, "exact potential is NULL");
    return mlp_stream(mlp, exact, cfg, tol, judge_every, ics, final_w, snaps, status, fallbacks, workspace,
                      workspace_bytes, stream);
}

}  // extern "C"
