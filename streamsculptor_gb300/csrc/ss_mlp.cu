// ss_mlp.cu — the learned force surrogate on CUDA cores: FP32 evaluation
// (potential and its analytic input gradient) and Sobolev training (value
// and force loss, differentiated through the input gradient) with Adam.
//
// Network: u (4) -> 128 -> 128 -> 128 -> 128 -> 1, SiLU after each hidden
// layer, u = affine(x, y, z, ln r).  With z_k = W_k a_{k-1} + b_k,
// a_k = s(z_k) (SiLU), y = w5 . a4 + b5, the input gradient is the backward
// chain
//   d4 = w5 * s'(z4),  d_{k-1} = (W_k^T d_k) * s'(z_{k-1}),  g = W1^T d1.
// Training differentiates L = w_v (Phi - Phi_t)^2 + w_f |grad Phi - g_t|^2
// through both the forward pass (value) and that chain (force):
//   dbar1 = W1 gbar,  ubar_k = dbar_k * s'(z_k),  sbar_k = dbar_k * u_k,
//   Wbar_{k+1} += d_{k+1} ubar_k^T,  dbar_{k+1} = W_{k+1} ubar_k,
//   w5bar += dbar4 * s'(z4),  sbar4 = dbar4 * w5,
// then the ordinary backward pass with the extra seeds sbar_k s''(z_k):
//   zbar_k = abar_k * s'(z_k) + sbar_k * s''(z_k),  Wbar_k += zbar_k a_{k-1}^T,
//   bbar_k += zbar_k,  abar_{k-1} = W_k^T zbar_k.
// Every matrix product is one launch of the tiled FP32 GEMM below (batch
// rows x 128 features, row-major); weight gradients use split-K with FP32
// atomics.  The tensor-core inference path lives in ss_mlp_stream.cu.

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "ss_common.cuh"
#include "ss_tcgen05.cuh"

namespace ssg {

static constexpr int MW = SS_MLP_WIDTH;  // 128
// packed parameter offsets (W[out][in])
static constexpr int64_t OFF_W1 = 0;
static constexpr int64_t OFF_B1 = OFF_W1 + MW * 4;
static constexpr int64_t OFF_W2 = OFF_B1 + MW;
static constexpr int64_t OFF_B2 = OFF_W2 + MW * MW;
static constexpr int64_t OFF_W3 = OFF_B2 + MW;
static constexpr int64_t OFF_B3 = OFF_W3 + MW * MW;
static constexpr int64_t OFF_W4 = OFF_B3 + MW;
static constexpr int64_t OFF_B4 = OFF_W4 + MW * MW;
static constexpr int64_t OFF_W5 = OFF_B4 + MW;
static constexpr int64_t OFF_B5 = OFF_W5 + MW;
static_assert(OFF_B5 + 1 == SS_MLP_NPARAM, "parameter packing");

struct MlpNorm {
    float c[4], s[4];  // u_i = (feature_i - s_i) c_i
    float out_scale, out_shift;
    const double* base;  // exact spherical part (ss_mlp.base), or NULL
    int base_n;
    double base_u0, base_du;
};

static MlpNorm norm_of(const ss_mlp* m) {
    MlpNorm n;
    for (int i = 0; i < 4; ++i) {
        n.c[i] = m->in_scale[i];
        n.s[i] = m->in_shift[i];
    }
    n.out_scale = m->out_scale;
    n.out_shift = m->out_shift;
    n.base = m->base;
    n.base_n = m->base_n;
    n.base_u0 = m->base_u0;
    n.base_du = m->base_du;
    return n;
}

// ------------------------------------------------------------- GEMM
// C[M,N] (=|+=) op(A)[M,K] op(B)[K,N] (+ bias[n]); row-major operands:
// A is [M,K] (lda) or, with TA, [K,M]; B is [K,N] (ldb) or, with TB, [N,K].
// 64 x 64 tiles, 16-deep K slices, 256 threads with 4 x 4 outputs each.
// ATOMIC: split-K over gridDim.z, accumulated with atomicAdd.
static constexpr int GB_M = 64, GB_N = 64, GB_K = 16;

template <bool TA, bool TB, bool ATOMIC>
__global__ void __launch_bounds__(256) gemm_kernel(int M, int N, int K, const float* __restrict__ A, int lda,
                                                   const float* __restrict__ B, int ldb, float* C, int ldc,
                                                   const float* __restrict__ bias, int kchunk) {
    __shared__ float As[GB_K][GB_M + 4];
    __shared__ float Bs[GB_K][GB_N + 4];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int m0 = blockIdx.y * GB_M, n0 = blockIdx.x * GB_N;
    const int kb = blockIdx.z * kchunk, ke = min(K, kb + kchunk);
    float acc[4][4] = {};
    for (int k0 = kb; k0 < ke; k0 += GB_K) {
        for (int e = threadIdx.x; e < GB_M * GB_K; e += 256) {
            int mm, kk;
            if (TA) { mm = e % GB_M; kk = e / GB_M; } else { kk = e % GB_K; mm = e / GB_K; }
            const int gm = m0 + mm, gk = k0 + kk;
            float v = 0.0f;
            if (gm < M && gk < ke) v = TA ? A[(int64_t)gk * lda + gm] : A[(int64_t)gm * lda + gk];
            As[kk][mm] = v;
        }
        for (int e = threadIdx.x; e < GB_N * GB_K; e += 256) {
            int nn, kk;
            if (TB) { kk = e % GB_K; nn = e / GB_K; } else { nn = e % GB_N; kk = e / GB_N; }
            const int gn = n0 + nn, gk = k0 + kk;
            float v = 0.0f;
            if (gn < N && gk < ke) v = TB ? B[(int64_t)gn * ldb + gk] : B[(int64_t)gk * ldb + gn];
            Bs[kk][nn] = v;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < GB_K; ++kk) {
            float a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                a[i] = As[kk][ty * 4 + i];
                b[i] = Bs[kk][tx * 4 + i];
            }
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int gm = m0 + ty * 4 + i;
        if (gm >= M) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int gn = n0 + tx * 4 + j;
            if (gn >= N) continue;
            float v = acc[i][j];
            if (ATOMIC) {
                atomicAdd(C + (int64_t)gm * ldc + gn, v);
            } else {
                if (bias) v += bias[gn];
                C[(int64_t)gm * ldc + gn] = v;
            }
        }
    }
}

// 1: the 128-wide training products on the tensor cores (tc_gemm below);
// 0: every product on the CUDA-core GEMM (ss_mlp_train_backend)
static int g_tc_train = 1;

template <bool TA, bool TB, bool ATOMIC>
static void tc_gemm(int M, int K, const float* A, int lda, const float* B, int ldb, float* C, int ldc,
                    const float* bias, int splits, cudaStream_t st);
static bool tc_ok(int N, int K, const float* A, int lda, const float* B, int ldb, const float* C, int ldc,
                  const float* bias);

template <bool TA, bool TB>
static void gemm(int M, int N, int K, const float* A, int lda, const float* B, int ldb, float* C, int ldc,
                 const float* bias, cudaStream_t st) {
    if (g_tc_train && tc_ok(N, K, A, lda, B, ldb, C, ldc, bias)) {
        tc_gemm<TA, TB, false>(M, K, A, lda, B, ldb, C, ldc, bias, 1, st);
        return;
    }
    dim3 grid((N + GB_N - 1) / GB_N, (M + GB_M - 1) / GB_M, 1);
    gemm_kernel<TA, TB, false><<<grid, 256, 0, st>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, K);
    count_launch();
}

// C += op(A) op(B), split over K (the batch) for the weight gradients.
template <bool TA, bool TB>
static void gemm_acc(int M, int N, int K, const float* A, int lda, const float* B, int ldb, float* C, int ldc,
                     cudaStream_t st) {
    if (g_tc_train && tc_ok(N, K, A, lda, B, ldb, C, ldc, nullptr)) {
        // split-K over the batch: K ranges of 128 (four chunks) per CTA
        tc_gemm<TA, TB, true>(M, K, A, lda, B, ldb, C, ldc, nullptr, (K + 127) / 128, st);
        return;
    }
    const int tiles = ((N + GB_N - 1) / GB_N) * ((M + GB_M - 1) / GB_M);
    int splits = (4 * 152 + tiles - 1) / tiles;
    int kchunk = (K + splits - 1) / splits;
    kchunk = (kchunk + GB_K - 1) / GB_K * GB_K;
    splits = (K + kchunk - 1) / kchunk;
    dim3 grid((N + GB_N - 1) / GB_N, (M + GB_M - 1) / GB_M, splits);
    gemm_kernel<TA, TB, true><<<grid, 256, 0, st>>>(M, N, K, A, lda, B, ldb, C, ldc, nullptr, kchunk);
    count_launch();
}

// ------------------------------------------ tensor-core GEMM (N = 128)
// C[M,128] (= acc + bias, or += acc by atomics for split-K) =
// op(A)[M,K] op(B)[K,128] with tcgen05.mma kind::tf32 (FP32 accumulation
// in TMEM).  Every FP32 operand is split into a TF32 head and remainder,
// a = a_h + a_l (a_h: a with its 13 low mantissa bits cleared, a_l = a - a_h
// exactly), and the product is a_h b_h + a_h b_l + a_l b_h: the dropped
// a_l b_l is 2^-22 relative, so the products stay near FP32 accuracy
// (about 1e-5 relative on the training gradient, where single TF32 MMAs,
// dropping 13 bits of every operand, give about 1e-3) while the tensor
// cores do the work.
// Operands as in the CUDA-core GEMM: A is [M,K] (lda) or, with TA, [K,M];
// B is [K,N] (ldb) or, with TB, [N,K] (C = A W^T with W[out][in]).  Both
// are staged K-major: an operand whose K is not the contiguous index is
// transposed on the way into shared memory.
// One CTA of 128 threads per 128-row tile of C (grid.x) and K range
// (grid.y); K in chunks of 32 staged in shared memory as K-major core
// matrices (8 rows x 4 elements, 128 bytes), element (r, k) of a 128 x 32
// chunk at byte (r/8) 1024 + (k/4) 128 + (r%8) 16 + (k%4) 4 (LBO 128,
// SBO 1024), double-buffered: the threads stage chunk c + 1 while the MMAs
// of chunk c run.  Warp w reads TMEM lanes 32w..32w+31 (rows of C).  A wait
// that runs out writes NaN into the CTA's part of C, so the failure reaches
// the loss.
constexpr int TC_THREADS = 128, TC_KC = 32;
constexpr uint32_t TC_OPER = 16384;            // one 128 x 32 FP32 chunk
constexpr uint32_t TC_BUF = 4 * TC_OPER;       // A_h, A_l, B_h, B_l
constexpr uint32_t TC_BAR = 2 * TC_BUF;        // 2 mbarriers
constexpr uint32_t TC_TMEM = TC_BAR + 16;      // TMEM base address
constexpr uint32_t TC_SMEM = TC_TMEM + 16 + 1024;  // + slack for the 1024-byte alignment

__device__ __forceinline__ uint32_t tc_off(int r, int k) {
    return (uint32_t)((r >> 3) * 1024 + (k >> 2) * 128 + (r & 7) * 16 + (k & 3) * 4);
}

__device__ __forceinline__ float tf32_head(float a) { return __uint_as_float(__float_as_uint(a) & 0xffffe000u); }

// One operand's 128 x 32 chunk in flight: rows [r0, r0 + 128) x K [k0,
// k0 + 32), 8 float4 per thread, loaded to registers first (tc_load) so the
// loads of chunk c + 1 overlap the MMAs of chunk c, then split into head and
// remainder and stored as core matrices (tc_put).  Rows at or past `rows`
// are zero.
struct TcRegs {
    float4 v[8];
};

template <bool T>
__device__ __forceinline__ void tc_load(TcRegs& g, const float* X, int ld, int r0, int rows, int k0) {
    const int t = threadIdx.x;
    if (!T) {
        // float4 along K: 8 consecutive threads take rows r..r+7 at one K
        // quad (conflict-free 16-byte stores), a warp 8 rows x 64 bytes
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int idx = t + TC_THREADS * i;
            const int r = ((idx >> 6) << 3) | (idx & 7), kq = (idx >> 3) & 7;
            g.v[i] = make_float4(0.f, 0.f, 0.f, 0.f);
            if (r0 + r < rows) g.v[i] = *reinterpret_cast<const float4*>(X + (int64_t)(r0 + r) * ld + k0 + 4 * kq);
        }
    } else {
        // X[k][r]: a 4 x 4 block per thread and pass (four float4 along r at
        // consecutive k), transposed in registers when stored
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            const int idx = t + TC_THREADS * i;
            const int rq = idx & 31, kq = idx >> 5;
            const int r = 4 * rq;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                float4& v = g.v[4 * i + j];
                v = make_float4(0.f, 0.f, 0.f, 0.f);
                const float* src = X + (int64_t)(k0 + 4 * kq + j) * ld + r0 + r;
                if (r0 + r + 3 < rows) {
                    v = *reinterpret_cast<const float4*>(src);
                } else {
                    if (r0 + r < rows) v.x = src[0];
                    if (r0 + r + 1 < rows) v.y = src[1];
                    if (r0 + r + 2 < rows) v.z = src[2];
                }
            }
        }
    }
}

__device__ __forceinline__ void tc_put4(uint8_t* hi, uint8_t* lo, uint32_t o, float4 w) {
    const float4 h = make_float4(tf32_head(w.x), tf32_head(w.y), tf32_head(w.z), tf32_head(w.w));
    *reinterpret_cast<float4*>(hi + o) = h;
    *reinterpret_cast<float4*>(lo + o) = make_float4(w.x - h.x, w.y - h.y, w.z - h.z, w.w - h.w);
}

template <bool T>
__device__ __forceinline__ void tc_put(const TcRegs& g, uint8_t* hi, uint8_t* lo) {
    const int t = threadIdx.x;
    if (!T) {
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int idx = t + TC_THREADS * i;
            const int r = ((idx >> 6) << 3) | (idx & 7), kq = (idx >> 3) & 7;
            tc_put4(hi, lo, tc_off(r, 4 * kq), g.v[i]);
        }
    } else {
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            const int idx = t + TC_THREADS * i;
            const int rq = idx & 31, kq = idx >> 5;
            const float4* v = g.v + 4 * i;
            tc_put4(hi, lo, tc_off(4 * rq, 4 * kq), make_float4(v[0].x, v[1].x, v[2].x, v[3].x));
            tc_put4(hi, lo, tc_off(4 * rq + 1, 4 * kq), make_float4(v[0].y, v[1].y, v[2].y, v[3].y));
            tc_put4(hi, lo, tc_off(4 * rq + 2, 4 * kq), make_float4(v[0].z, v[1].z, v[2].z, v[3].z));
            tc_put4(hi, lo, tc_off(4 * rq + 3, 4 * kq), make_float4(v[0].w, v[1].w, v[2].w, v[3].w));
        }
    }
}

template <bool TA, bool TB, bool ATOMIC>
__global__ void __launch_bounds__(TC_THREADS, 1) tc_gemm_kernel(int M, int K, const float* __restrict__ A, int lda,
                                                                const float* __restrict__ B, int ldb, float* C,
                                                                int ldc, const float* __restrict__ bias, int kchunk) {
    extern __shared__ uint8_t tc_dyn[];
    uint8_t* sm = (uint8_t*)(((uintptr_t)tc_dyn + 1023) & ~(uintptr_t)1023);
    const int t = threadIdx.x, w = t >> 5;
    const int m0 = blockIdx.x * 128;
    const int kb = blockIdx.y * kchunk, ke = min(K, kb + kchunk);
    const int nc = ke > kb ? (ke - kb) / TC_KC : 0;
    const uint32_t bar0 = smem_u32(sm + TC_BAR), base = smem_u32(sm);
    if (t == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar0), "r"(1));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar0 + 8), "r"(1));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (w == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(sm + TC_TMEM)),
                     "r"(128));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    TcRegs ra, rb;
    if (nc > 0) {
        tc_load<TA>(ra, A, lda, m0, M, kb);
        tc_load<!TB>(rb, B, ldb, 0, 128, kb);
        tc_put<TA>(ra, sm, sm + TC_OPER);
        tc_put<!TB>(rb, sm + 2 * TC_OPER, sm + 3 * TC_OPER);
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(sm + TC_TMEM);
    const uint32_t id = idesc_tf32();
    bool ok = true;
    for (int c = 0; c < nc; ++c) {
        const uint32_t b = c & 1, buf = base + b * TC_BUF;
        fence_async_smem();  // this thread's staged chunk -> the tensor cores' proxy
        fence_before();
        __syncthreads();
        fence_after();
        if (t == 0) {
#pragma unroll
            for (int kk = 0; kk < TC_KC / 8; ++kk) {
                const uint64_t ah = smem_desc(buf + kk * 256, 128, 1024);
                const uint64_t al = smem_desc(buf + TC_OPER + kk * 256, 128, 1024);
                const uint64_t bh = smem_desc(buf + 2 * TC_OPER + kk * 256, 128, 1024);
                const uint64_t bl = smem_desc(buf + 3 * TC_OPER + kk * 256, 128, 1024);
                mma_tf32(tmem, ah, bh, id, (c > 0 || kk > 0) ? 1u : 0u);
                mma_tf32(tmem, ah, bl, id, 1u);
                mma_tf32(tmem, al, bh, id, 1u);
            }
            mma_commit(bar0 + 8 * b);
        }
        if (c + 1 < nc) {
            const uint32_t b1 = (c + 1) & 1;
            // chunk c + 1 into registers while the MMAs run; buffer b1 last
            // fed chunk c - 1: wait for its MMAs before storing
            tc_load<TA>(ra, A, lda, m0, M, kb + (c + 1) * TC_KC);
            tc_load<!TB>(rb, B, ldb, 0, 128, kb + (c + 1) * TC_KC);
            if (c >= 1) ok = ok && mbar_wait(bar0 + 8 * b1, (uint32_t)(((c - 1) >> 1) & 1));
            if (__syncthreads_or(!ok)) {
                ok = false;
                break;
            }
            uint8_t* nb = sm + b1 * TC_BUF;
            tc_put<TA>(ra, nb, nb + TC_OPER);
            tc_put<!TB>(rb, nb + 2 * TC_OPER, nb + 3 * TC_OPER);
        }
    }
    if (nc > 0 && ok) ok = mbar_wait(bar0 + 8 * ((nc - 1) & 1), (uint32_t)(((nc - 1) >> 1) & 1));
    ok = !__syncthreads_or(!ok);
    fence_after();
    const int row = m0 + 32 * w + (t & 31);
    const float qnan = __int_as_float(0x7fc00000);
    if (nc > 0) {
#pragma unroll 1
        for (int q = 0; q < 4; ++q) {
            uint32_t r[32];
            SS_TMEM_LD32(r, tmem + ((uint32_t)(32 * w) << 16) + 32 * q);
            tmem_wait_ld();
            if (row < M) {
                float* out = C + (int64_t)row * ldc + 32 * q;
#pragma unroll
                for (int j = 0; j < 32; j += 4) {
                    float4 v = ok ? make_float4(__uint_as_float(r[j]), __uint_as_float(r[j + 1]),
                                                __uint_as_float(r[j + 2]), __uint_as_float(r[j + 3]))
                                  : make_float4(qnan, qnan, qnan, qnan);
                    if (ATOMIC) {
                        atomicAdd(reinterpret_cast<float4*>(out + j), v);  // one vector atomic (sm_90 and later)
                    } else {
                        if (bias) {
                            const float4 bb = *reinterpret_cast<const float4*>(bias + 32 * q + j);
                            v.x += bb.x;
                            v.y += bb.y;
                            v.z += bb.z;
                            v.w += bb.w;
                        }
                        *reinterpret_cast<float4*>(out + j) = v;
                    }
                }
            }
        }
    }
    if (!ok && t == 0) {
        // give the outstanding commits a bounded wait before TMEM is released
        mbar_wait(bar0, 0u);
        mbar_wait(bar0 + 8, 0u);
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (w == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(128));
}

// Whether a product can take the tensor-core GEMM: N = 128, K a multiple of
// 32, 16-byte aligned operands and leading dimensions.
static bool tc_ok(int N, int K, const float* A, int lda, const float* B, int ldb, const float* C, int ldc,
                  const float* bias) {
    auto al = [](const void* p) { return ((uintptr_t)p & 15) == 0; };
    return N == 128 && K > 0 && K % TC_KC == 0 && lda % 4 == 0 && ldb % 4 == 0 && ldc % 4 == 0 && al(A) && al(B) &&
           al(C) && (bias == nullptr || al(bias));
}

template <bool TA, bool TB, bool ATOMIC>
static void tc_gemm(int M, int K, const float* A, int lda, const float* B, int ldb, float* C, int ldc,
                    const float* bias, int splits, cudaStream_t st) {
    static bool attr[64] = {};  // the shared-memory opt-in, once per device
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && !attr[dev]) {
        cudaFuncSetAttribute(tc_gemm_kernel<TA, TB, ATOMIC>, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM);
        attr[dev] = true;
    }
    int kchunk = (K + splits - 1) / splits;
    kchunk = (kchunk + TC_KC - 1) / TC_KC * TC_KC;
    splits = (K + kchunk - 1) / kchunk;
    dim3 grid((M + 127) / 128, splits);
    tc_gemm_kernel<TA, TB, ATOMIC><<<grid, TC_THREADS, TC_SMEM, st>>>(M, K, A, lda, B, ldb, C, ldc, bias, kchunk);
    count_launch();
}

// ------------------------------------------------------ elementwise
__device__ __forceinline__ void silu3(float z, float& a, float& s1, float& s2) {
    const float sg = 1.0f / (1.0f + __expf(-z));
    a = z * sg;
    s1 = sg * (1.0f + z * (1.0f - sg));
    s2 = sg * (1.0f - sg) * (2.0f + z * (1.0f - 2.0f * sg));
}

// A = s(Z), S = s'(Z), P = s''(Z) (P may be NULL); Z is overwritten by A.
__global__ void silu_kernel(float* Z, float* S, float* P, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float a, s1, s2;
    silu3(Z[i], a, s1, s2);
    Z[i] = a;
    S[i] = s1;
    if (P) P[i] = s2;
}

// features u [B,4] and 1/r^2 from positions (FP32 or FP64 input)
template <class X>
__global__ void features_kernel(const X* __restrict__ x, int64_t B, MlpNorm nm, float* u, float* ir2) {
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    const double p0 = (double)x[3 * b], p1 = (double)x[3 * b + 1], p2 = (double)x[3 * b + 2];
    const double r2 = p0 * p0 + p1 * p1 + p2 * p2;
    u[4 * b + 0] = (float)((p0 - nm.s[0]) * nm.c[0]);
    u[4 * b + 1] = (float)((p1 - nm.s[1]) * nm.c[1]);
    u[4 * b + 2] = (float)((p2 - nm.s[2]) * nm.c[2]);
    u[4 * b + 3] = (float)((0.5 * log(r2) - nm.s[3]) * nm.c[3]);
    ir2[b] = (float)(1.0 / r2);
}

// D4 = S4 * w5 (row broadcast)
__global__ void d4_kernel(const float* S4, const float* w5, float* D4, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    D4[i] = S4[i] * w5[i % MW];
}

// X *= S (in place)
__global__ void mul_kernel(float* X, const float* S, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    X[i] *= S[i];
}

// Ubar = Dbar * S, Sbar = Dbar * U
__global__ void split_kernel(const float* Dbar, const float* S, const float* U, float* Ubar, float* Sbar, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Ubar[i] = Dbar[i] * S[i];
    Sbar[i] = Dbar[i] * U[i];
}

// Zbar = Abar * S + Sbar * P (Abar overwritten by Zbar)
__global__ void zbar_kernel(float* Abar, const float* S, const float* Sbar, const float* P, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Abar[i] = Abar[i] * S[i] + Sbar[i] * P[i];
}

// Phi and grad Phi per point from the last activations and the input
// gradient g [B,4].
__global__ void eval_out_kernel(const float* A4, const float* w5, const float* b5, const float* g, const float* ir2,
                                const double* x, int64_t B, MlpNorm nm, double* phi, double* grad) {
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    // the exact spherical part, FP64
    double f0 = 0.0, fu = 0.0, r2 = 1.0;
    if (nm.base) {
        r2 = x[3 * b] * x[3 * b] + x[3 * b + 1] * x[3 * b + 1] + x[3 * b + 2] * x[3 * b + 2];
        base_spline<double, double>(nm.base, nm.base_n, nm.base_u0, nm.base_du, 1.0 / nm.base_du, 0.5 * log(r2), f0,
                                    fu);
    }
    if (phi) {
        float y = b5[0];
        for (int j = 0; j < MW; ++j) y = fmaf(A4[b * MW + j], w5[j], y);
        phi[b] = (double)nm.out_scale * y + nm.out_shift + f0;
    }
    if (grad) {
        const float* gb = g + 4 * b;
        for (int j = 0; j < 3; ++j)
            grad[3 * b + j] = (double)nm.out_scale * (gb[j] * nm.c[j] + gb[3] * nm.c[3] * (float)x[3 * b + j] * ir2[b]) +
                              fu / r2 * x[3 * b + j];
    }
}

// Loss of each sample; seeds ybar [B] and gbar [B,4]; accumulates loss[0..1].
// One warp per sample: the lanes read the sample's 128 activations
// coalesced for y = w5 . a4 and reduce it with shuffles; lane 0 does the rest.
constexpr int LOSS_ROWS = 8;  // samples (warps) per block
__global__ void loss_kernel(const float* A4, const float* prm, const float* g, const float* ir2, const float* x,
                            const float* phi_t, const float* g_t, const float* w_val, const float* w_force,
                            int64_t B, MlpNorm nm, float* ybar, float* gbar, float* loss) {
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    const int64_t b = (int64_t)blockIdx.x * LOSS_ROWS + w;
    float lv = 0.0f, lf = 0.0f;
    if (b < B) {
        const float* w5 = prm + OFF_W5;
        float y = 0.0f;
#pragma unroll
        for (int j = l; j < MW; j += 32) y = fmaf(A4[b * MW + j], w5[j], y);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) y += __shfl_xor_sync(0xffffffffu, y, o);
        if (l == 0) {
            y += prm[OFF_B5];
            const float ev = nm.out_scale * y + nm.out_shift - phi_t[b];
            lv = w_val[b] * ev * ev;
            ybar[b] = 2.0f * w_val[b] * ev * nm.out_scale;
            const float* gb = g + 4 * b;
            float e[3], ex = 0.0f;
            for (int j = 0; j < 3; ++j) {
                const float pred = nm.out_scale * (gb[j] * nm.c[j] + gb[3] * nm.c[3] * x[3 * b + j] * ir2[b]);
                e[j] = pred - g_t[3 * b + j];
                lf += e[j] * e[j];
                ex += e[j] * x[3 * b + j];
            }
            lf *= w_force[b];
            const float k = 2.0f * w_force[b] * nm.out_scale;
            for (int j = 0; j < 3; ++j) gbar[4 * b + j] = k * nm.c[j] * e[j];
            gbar[4 * b + 3] = k * nm.c[3] * ex * ir2[b];
        }
    }
    // block reduction of the two loss parts (lane 0 of each warp holds its sample's)
    __shared__ float red[2][LOSS_ROWS];
    if (l == 0) {
        red[0][w] = lv;
        red[1][w] = lf;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float a = 0.0f, c = 0.0f;
        for (int i = 0; i < LOSS_ROWS; ++i) {
            a += red[0][i];
            c += red[1][i];
        }
        atomicAdd(loss, a);
        atomicAdd(loss + 1, c);
    }
}

// rows per block of the column sums below (one thread per feature): short
// loops and many blocks, the partial sums added with atomics
constexpr int SUM_ROWS = 8;

// Zbar4 = ybar w5 * S4 + Sbar4 * P4, Sbar4 = Dbar4 * w5 (computed here);
// accumulates w5bar += Dbar4 * S4 + ybar A4 (column sums) and b5bar.
__global__ void top_kernel(const float* Dbar4, const float* S4, const float* P4, const float* A4, const float* ybar,
                           const float* w5, int64_t B, float* Zbar4, float* w5bar, float* b5bar) {
    const int j = threadIdx.x;  // feature (blockDim.x == 128)
    const int64_t r0 = (int64_t)blockIdx.x * SUM_ROWS;
    float acc = 0.0f, accb = 0.0f;
    for (int64_t b = r0; b < r0 + SUM_ROWS && b < B; ++b) {
        const int64_t i = b * MW + j;
        const float sb = Dbar4[i] * w5[j];
        Zbar4[i] = ybar[b] * w5[j] * S4[i] + sb * P4[i];
        acc += Dbar4[i] * S4[i] + ybar[b] * A4[i];
        if (j == 0) accb += ybar[b];
    }
    atomicAdd(w5bar + j, acc);
    if (j == 0) atomicAdd(b5bar, accb);
}

// bbar[j] += sum_b Zbar[b][j]
__global__ void colsum_kernel(const float* Z, int64_t B, float* out) {
    const int j = threadIdx.x;
    const int64_t r0 = (int64_t)blockIdx.x * SUM_ROWS;
    float acc = 0.0f;
    for (int64_t b = r0; b < r0 + SUM_ROWS && b < B; ++b) acc += Z[b * MW + j];
    atomicAdd(out + j, acc);
}

__global__ void adam_kernel(float* p, const float* g, float* m, float* v, int64_t n, float lr, float b1, float b2,
                            float eps, float c1, float c2) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
}

static inline unsigned blocks(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

// ------------------------------------------------- forward + input gradient
// Buffers (row-major, B rows): A1..A4 [B,128] (activations), S1..S4 (s'),
// P1..P4 (s'', training only), D1..D4 (input-gradient chain: D_k = U_k * S_k,
// U_k = D_{k+1} W_{k+1}), g [B,4].
struct MlpBufs {
    float *u, *ir2;
    float *A[5], *S[5], *P[5], *D[5], *U[5];  // index 1..4
    float* g;
};

static void forward_and_input_grad(const float* prm, int B, const MlpBufs& w, bool keep_u, cudaStream_t st) {
    const int64_t n = (int64_t)B * MW;
    const float* Wk[5] = {nullptr, prm + OFF_W1, prm + OFF_W2, prm + OFF_W3, prm + OFF_W4};
    const float* bk[5] = {nullptr, prm + OFF_B1, prm + OFF_B2, prm + OFF_B3, prm + OFF_B4};
    // z1 = u W1^T + b1 (K = 4), then z_k = a_{k-1} W_k^T + b_k
    gemm<false, true>(B, MW, 4, w.u, 4, Wk[1], 4, w.A[1], MW, bk[1], st);
    silu_kernel<<<blocks(n, 256), 256, 0, st>>>(w.A[1], w.S[1], w.P[1], n);
    count_launch();
    for (int k = 2; k <= 4; ++k) {
        gemm<false, true>(B, MW, MW, w.A[k - 1], MW, Wk[k], MW, w.A[k], MW, bk[k], st);
        silu_kernel<<<blocks(n, 256), 256, 0, st>>>(w.A[k], w.S[k], w.P[k], n);
        count_launch();
    }
    // d4 = w5 * s'(z4); d_{k-1} = (d_k W_k) * s'(z_{k-1}); g = d1 W1
    d4_kernel<<<blocks(n, 256), 256, 0, st>>>(w.S[4], prm + OFF_W5, w.D[4], n);
    count_launch();
    for (int k = 4; k >= 2; --k) {
        float* U = keep_u ? w.U[k - 1] : w.D[k - 1];
        gemm<false, false>(B, MW, MW, w.D[k], MW, Wk[k], MW, U, MW, nullptr, st);
        if (keep_u) {
            // D_{k-1} = U_{k-1} * S_{k-1}, keeping U_{k-1}
            cudaMemcpyAsync(w.D[k - 1], U, n * sizeof(float), cudaMemcpyDeviceToDevice, st);
        }
        mul_kernel<<<blocks(n, 256), 256, 0, st>>>(w.D[k - 1], w.S[k - 1], n);
        count_launch();
    }
    gemm<false, false>(B, 4, MW, w.D[1], MW, Wk[1], 4, w.g, 4, nullptr, st);
}

static constexpr int64_t EVAL_CHUNK = 1 << 14;

static MlpBufs carve(float* base, int64_t B, bool train, float** rest) {
    MlpBufs w{};
    float* p = base;
    auto take = [&](int64_t cols) {
        float* q = p;
        p += ((B * cols + 63) / 64) * 64;
        return q;
    };
    w.u = take(4);
    w.ir2 = take(1);
    w.g = take(4);
    for (int k = 1; k <= 4; ++k) {
        w.A[k] = take(MW);
        w.S[k] = take(MW);
        w.D[k] = take(MW);
        w.P[k] = train ? take(MW) : nullptr;
        w.U[k] = (train && k < 4) ? take(MW) : nullptr;
    }
    if (rest) *rest = p;
    return w;
}

static int64_t bufs_bytes(int64_t B, bool train) {
    // each buffer rounded up to 64 floats
    const int64_t per = train ? 9 + 5 + (12 + 4 + 3 + 7) * MW : 9 + 12 * MW;
    return (per * B + 64 * 40) * (int64_t)sizeof(float) + 256;
}

}  // namespace ssg

using namespace ssg;

extern "C" {

int64_t ss_mlp_eval_workspace_bytes(int64_t n) {
    if (n < 0) return set_error(SS_ERR_INVALID_ARGUMENT, "n < 0");
    return bufs_bytes(n < EVAL_CHUNK ? n : EVAL_CHUNK, false);
}

int ss_mlp_eval(const ss_mlp* mlp, const double* xyz, int64_t n, double* phi, double* grad, void* workspace,
                int64_t workspace_bytes, void* stream) {
    SS_CHECK_ARG(mlp != nullptr && mlp->params != nullptr, "mlp or its params is NULL");
    SS_CHECK_ARG(n >= 0, "n < 0");
    if (n == 0) return SS_OK;
    SS_CHECK_ARG(xyz != nullptr, "xyz is NULL");
    SS_CHECK_ARG(mlp->base == nullptr || (mlp->base_n >= 2 && mlp->base_n <= SS_MLP_BASE_MAX && mlp->base_du > 0.0),
                 "mlp base table needs 2 <= base_n <= %d knots and base_du > 0", SS_MLP_BASE_MAX);
    const int64_t need = ss_mlp_eval_workspace_bytes(n);
    if (workspace == nullptr || workspace_bytes < need)
        return set_error(SS_ERR_WORKSPACE, "workspace of %lld bytes needed", (long long)need);
    cudaStream_t st = (cudaStream_t)stream;
    const MlpNorm nm = norm_of(mlp);
    const float* prm = mlp->params;
    for (int64_t b0 = 0; b0 < n; b0 += EVAL_CHUNK) {
        const int B = (int)((n - b0) < EVAL_CHUNK ? (n - b0) : EVAL_CHUNK);
        MlpBufs w = carve((float*)workspace, B, false, nullptr);
        features_kernel<double><<<blocks(B, 256), 256, 0, st>>>(xyz + 3 * b0, B, nm, w.u, w.ir2);
        SS_LAUNCH_CHECK();
        forward_and_input_grad(prm, B, w, false, st);
        eval_out_kernel<<<blocks(B, 128), 128, 0, st>>>(w.A[4], prm + OFF_W5, prm + OFF_B5, w.g, w.ir2, xyz + 3 * b0, B,
                                                         nm, phi ? phi + b0 : nullptr, grad ? grad + 3 * b0 : nullptr);
        SS_LAUNCH_CHECK();
    }
    return SS_OK;
}

int64_t ss_mlp_train_workspace_bytes(int64_t batch) {
    if (batch <= 0) return set_error(SS_ERR_INVALID_ARGUMENT, "batch <= 0");
    return bufs_bytes(batch, true);
}

}  // extern "C"

namespace ssg {

// The body of ss_mlp_loss_grad (arguments checked by the callers).
static int loss_grad_impl(const MlpNorm& nm, const float* prm, const float* x, const float* phi_t, const float* g_t,
                          const float* w_val, const float* w_force, int64_t batch, float* loss, float* grad,
                          void* workspace, cudaStream_t st) {
    const int B = (int)batch;
    const int64_t n = (int64_t)B * MW;
    float* rest = nullptr;
    MlpBufs w = carve((float*)workspace, B, true, &rest);
    auto take = [&](int64_t cols) {
        float* q = rest;
        rest += ((B * cols + 63) / 64) * 64;
        return q;
    };
    float* ybar = take(1);
    float* gbar = take(4);
    float* Dbar = take(MW);
    float* Ubar = take(MW);
    float* Sbar[5] = {nullptr, take(MW), take(MW), take(MW), take(MW)};
    float* Zbar = take(MW);
    SS_CUDA_TRY(cudaMemsetAsync(grad, 0, SS_MLP_NPARAM * sizeof(float), st));
    SS_CUDA_TRY(cudaMemsetAsync(loss, 0, 2 * sizeof(float), st));
    features_kernel<float><<<blocks(B, 256), 256, 0, st>>>(x, B, nm, w.u, w.ir2);
    SS_LAUNCH_CHECK();
    forward_and_input_grad(prm, B, w, true, st);
    loss_kernel<<<blocks(B, LOSS_ROWS), 32 * LOSS_ROWS, 0, st>>>(w.A[4], prm, w.g, w.ir2, x, phi_t, g_t, w_val, w_force, B, nm, ybar,
                                                gbar, loss);
    SS_LAUNCH_CHECK();
    const float* Wk[5] = {nullptr, prm + OFF_W1, prm + OFF_W2, prm + OFF_W3, prm + OFF_W4};
    float* gW[5] = {nullptr, grad + OFF_W1, grad + OFF_W2, grad + OFF_W3, grad + OFF_W4};
    float* gb[5] = {nullptr, grad + OFF_B1, grad + OFF_B2, grad + OFF_B3, grad + OFF_B4};
    // reverse through the input-gradient chain: W1bar += D1^T gbar, Dbar1 = gbar W1^T
    gemm_acc<true, false>(MW, 4, B, w.D[1], MW, gbar, 4, gW[1], 4, st);
    gemm<false, true>(B, MW, 4, gbar, 4, Wk[1], 4, Dbar, MW, nullptr, st);
    for (int k = 1; k <= 3; ++k) {
        // Ubar_k = Dbar_k * S_k, Sbar_k = Dbar_k * U_k
        split_kernel<<<blocks(n, 256), 256, 0, st>>>(Dbar, w.S[k], w.U[k], Ubar, Sbar[k], n);
        SS_LAUNCH_CHECK();
        // W_{k+1}bar += D_{k+1}^T Ubar_k ; Dbar_{k+1} = Ubar_k W_{k+1}^T
        gemm_acc<true, false>(MW, MW, B, w.D[k + 1], MW, Ubar, MW, gW[k + 1], MW, st);
        gemm<false, true>(B, MW, MW, Ubar, MW, Wk[k + 1], MW, Dbar, MW, nullptr, st);
    }
    // top: Sbar4 = Dbar4 * w5, w5bar, b5bar, Zbar4
    top_kernel<<<blocks(B, SUM_ROWS), MW, 0, st>>>(Dbar, w.S[4], w.P[4], w.A[4], ybar, prm + OFF_W5, B, Zbar,
                                             grad + OFF_W5, grad + OFF_B5);
    SS_LAUNCH_CHECK();
    for (int k = 4; k >= 1; --k) {
        // Zbar_k ready: W_k bar += Zbar_k^T a_{k-1}, b_k bar += colsum(Zbar_k)
        const float* Aprev = k == 1 ? w.u : w.A[k - 1];
        const int kin = k == 1 ? 4 : MW;
        gemm_acc<true, false>(MW, kin, B, Zbar, MW, Aprev, kin, gW[k], kin, st);
        colsum_kernel<<<blocks(B, SUM_ROWS), MW, 0, st>>>(Zbar, B, gb[k]);
        SS_LAUNCH_CHECK();
        if (k == 1) break;
        // Abar_{k-1} = Zbar_k W_k ; Zbar_{k-1} = Abar * S_{k-1} + Sbar_{k-1} * P_{k-1}
        gemm<false, false>(B, MW, MW, Zbar, MW, Wk[k], MW, Dbar, MW, nullptr, st);
        zbar_kernel<<<blocks(n, 256), 256, 0, st>>>(Dbar, w.S[k - 1], Sbar[k - 1], w.P[k - 1], n);
        SS_LAUNCH_CHECK();
        float* t = Zbar;
        Zbar = Dbar;
        Dbar = t;
    }
    return SS_OK;
}

// One training batch gathered from the training set by sample index.
__global__ void gather_batch_kernel(const float* __restrict__ x, const float* __restrict__ phi,
                                    const float* __restrict__ g, const float* __restrict__ wv,
                                    const float* __restrict__ wf, const int32_t* __restrict__ idx, int64_t B,
                                    float* xb, float* pb, float* gb, float* wvb, float* wfb) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B) return;
    const int64_t j = idx[i];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        xb[3 * i + c] = x[3 * j + c];
        gb[3 * i + c] = g[3 * j + c];
    }
    pb[i] = phi[j];
    wvb[i] = wv[j];
    wfb[i] = wf[j];
}

// the gathered batch (x, phi, g, w_val, w_force), the gradient and the loss
// ahead of the training buffers in the fit workspace, 256-byte aligned each
static int64_t fit_head_floats(int64_t B) {
    auto up = [](int64_t f) { return (f + 63) / 64 * 64; };
    return up(3 * B) + up(B) + up(3 * B) + up(B) + up(B) + up(SS_MLP_NPARAM) + 64;
}

}  // namespace ssg

extern "C" {

int ss_mlp_loss_grad(const ss_mlp* mlp, const float* x, const float* phi_t, const float* g_t, const float* w_val,
                     const float* w_force, int64_t batch, float* loss, float* grad, void* workspace,
                     int64_t workspace_bytes, void* stream) {
    SS_CHECK_ARG(mlp != nullptr && mlp->params != nullptr, "mlp or its params is NULL");
    SS_CHECK_ARG(batch > 0 && batch <= (1 << 24), "batch outside [1, 2^24]");
    SS_CHECK_ARG(x && phi_t && g_t && w_val && w_force && loss && grad, "NULL buffer");
    const int64_t need = ss_mlp_train_workspace_bytes(batch);
    if (workspace == nullptr || workspace_bytes < need)
        return set_error(SS_ERR_WORKSPACE, "workspace of %lld bytes needed", (long long)need);
    return loss_grad_impl(norm_of(mlp), mlp->params, x, phi_t, g_t, w_val, w_force, batch, loss, grad, workspace,
                          (cudaStream_t)stream);
}

int64_t ss_mlp_fit_workspace_bytes(int64_t batch) {
    if (batch <= 0 || batch > (1 << 24)) return set_error(SS_ERR_INVALID_ARGUMENT, "batch outside [1, 2^24]");
    return fit_head_floats(batch) * (int64_t)sizeof(float) + bufs_bytes(batch, true);
}

int ss_mlp_fit(const ss_mlp* mlp, float* params, const float* x, const float* phi_t, const float* g_t,
               const float* w_val, const float* w_force, int64_t n, const int32_t* order, int64_t batch,
               int64_t steps, float lr, float lr_min, float beta1, float beta2, float eps, float* m, float* v,
               float* loss_log, void* workspace, int64_t workspace_bytes, void* stream) {
    SS_CHECK_ARG(mlp != nullptr && params != nullptr, "mlp or params is NULL");
    SS_CHECK_ARG(n > 0 && n <= INT32_MAX, "n outside [1, 2^31)");
    SS_CHECK_ARG(batch > 0 && batch <= (1 << 24), "batch outside [1, 2^24]");
    SS_CHECK_ARG(steps >= 0, "steps < 0");
    SS_CHECK_ARG(x && phi_t && g_t && w_val && w_force && order && m && v, "NULL buffer");
    SS_CHECK_ARG(mlp->base == nullptr || (mlp->base_n >= 2 && mlp->base_n <= SS_MLP_BASE_MAX && mlp->base_du > 0.0),
                 "mlp base table needs 2 <= base_n <= %d knots and base_du > 0", SS_MLP_BASE_MAX);
    const int64_t need = ss_mlp_fit_workspace_bytes(batch);
    if (workspace == nullptr || workspace_bytes < need)
        return set_error(SS_ERR_WORKSPACE, "workspace of %lld bytes needed", (long long)need);
    if (steps == 0) return SS_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const MlpNorm nm = norm_of(mlp);
    auto up = [](int64_t f) { return (f + 63) / 64 * 64; };
    float* p = static_cast<float*>(workspace);
    float* xb = p;
    float* pb = xb + up(3 * batch);
    float* gb = pb + up(batch);
    float* wvb = gb + up(3 * batch);
    float* wfb = wvb + up(batch);
    float* grad = wfb + up(batch);
    float* loss_tmp = grad + up(SS_MLP_NPARAM);
    void* train_ws = static_cast<void*>(p + fit_head_floats(batch));
    for (int64_t s = 0; s < steps; ++s) {
        gather_batch_kernel<<<blocks(batch, 256), 256, 0, st>>>(x, phi_t, g_t, w_val, w_force, order + s * batch, batch,
                                                                xb, pb, gb, wvb, wfb);
        SS_LAUNCH_CHECK();
        const int rc = loss_grad_impl(nm, params, xb, pb, gb, wvb, wfb, batch, loss_log ? loss_log + 2 * s : loss_tmp,
                                      grad, train_ws, st);
        if (rc) return rc;
        // cosine decay from lr to lr_min over the run; bias corrections of step s + 1
        const double lr_s = (double)lr_min + 0.5 * ((double)lr - (double)lr_min) *
                                                 (1.0 + std::cos(M_PI * (double)s / (double)std::max<int64_t>(steps - 1, 1)));
        const float c1 = (float)(1.0 / (1.0 - std::pow((double)beta1, (double)(s + 1))));
        const float c2 = (float)(1.0 / (1.0 - std::pow((double)beta2, (double)(s + 1))));
        adam_kernel<<<blocks(SS_MLP_NPARAM, 256), 256, 0, st>>>(params, grad, m, v, SS_MLP_NPARAM, (float)lr_s, beta1,
                                                                 beta2, eps, c1, c2);
        SS_LAUNCH_CHECK();
    }
    return SS_OK;
}

int ss_mlp_train_backend(int tensor_cores) {
    const int prev = g_tc_train;
    if (tensor_cores == 0 || tensor_cores == 1) g_tc_train = tensor_cores;
    return prev;
}

int ss_mlp_adam(float* params, const float* grad, float* m, float* v, int64_t n, int64_t step, float lr, float beta1,
                float beta2, float eps, void* stream) {
    SS_CHECK_ARG(params && grad && m && v, "NULL buffer");
    SS_CHECK_ARG(n > 0 && step >= 1, "need n > 0 and step >= 1");
    const float c1 = (float)(1.0 / (1.0 - std::pow((double)beta1, (double)step)));
    const float c2 = (float)(1.0 / (1.0 - std::pow((double)beta2, (double)step)));
    adam_kernel<<<blocks(n, 256), 256, 0, (cudaStream_t)stream>>>(params, grad, m, v, n, lr, beta1, beta2, eps, c1, c2);
    SS_LAUNCH_CHECK();
    return SS_OK;
}

}  // extern "C"
