// ss_stream.cu — the hot path: every released star integrated from its
// release step to the end with fixed-step Dormand-Prince 5(4), force fused
// into the stage loop, state and stages in registers.
//
// Reference: Potential.gen_stream_vmapped / gen_stream_scan (main.py:312-368)
// integrate particle i (lead and trail) from ts[i] to ts[-1] through
// integrate_orbit (main.py:125-163); gen_stream_vmapped_Chen25
// (streamhelpers.py:491-543) adds the moving progenitor (a
// TimeDepTranslatingPotential on a cubic spline of the progenitor orbit);
// gen_stream_vmapped_with_pert (streamhelpers.py:89-146) adds subhalos.
//
// Layout: one thread per particle (two for stream_f32k2_kernel, ss_stream2.cuh,
// the FP32 form for compiled compositions; one warp per potential component
// for stream_f64_split_kernel, the FP64 form of runs too small to occupy the
// GPU's schedulers); particles are ordered by release (release
// r owns particles [r*ppr, (r+1)*ppr)), so the earliest (longest) particles
// sit in the lowest blocks and are scheduled first.  A warp runs in global
// lock-step from its earliest start step: lanes released later idle until
// their release step, so every active lane evaluates the same stage time and
// the track / subhalo table reads are warp-uniform broadcasts.
//
// Two precisions:
//   ss_stream_f64   FP64 state, stages and force (parity path).
//   ss_stream_f32k  FP32 stages and force; position and velocity kept as
//                   compensated hi+lo float pairs; the increments are formed
//                   as h*v_hi (exact two-product) plus small corrections, so
//                   float rounding of the tableau touches only second-order
//                   terms.  Time and release bookkeeping are integer/FP64 and
//                   happen outside the step loop; the progenitor track and
//                   subhalo lines are pre-tabulated in FP32 (workspace).

#include <cuda_runtime.h>

#include <cmath>
#include <type_traits>

#include "ss_stream.cuh"
#include "ss_stream2.cuh"

namespace ssg {

// The FP64 stream kernel (its body, stream_f64_body, is in ss_stream.cuh).
// The analytic compositions fit the compiler's default register budget for
// 64-thread blocks without spills; the expansion and the generic
// composition need their larger register sets (one block per SM at least).
template <class C>
__global__ void __launch_bounds__(F64_BLOCK) stream_f64_kernel(PotDev<double> P, StreamArgs a) {
    stream_f64_body<C>(P, a);
}
template <>
__global__ void __launch_bounds__(F64_BLOCK, 1) stream_f64_kernel<GenericComp>(PotDev<double> P, StreamArgs a) {
    stream_f64_body<GenericComp>(P, a);
}
template <>
__global__ void __launch_bounds__(F64_BLOCK, 1) stream_f64_kernel<CompSHExp>(PotDev<double> P, StreamArgs a) {
    stream_f64_body<CompSHExp>(P, a);
}

// The component-split FP64 kernel for small runs (stream_f64_split_body).
template <class C>
__global__ void __launch_bounds__(32 * C::n) stream_f64_split_kernel(PotDev<double> P, StreamArgs a) {
    stream_f64_split_body<C>(P, a);
}

// Track positions at every stage time of the run, FP64 Hermite -> a hi/lo
// float pair (two float4).  Slot 5n + s holds c(t0 + (n + c_s) dt) for
// c = {0, 1/5, 3/10, 4/5, 8/9}; slot 5 n_steps holds c(t0 + n_steps dt).
__global__ void track_table_kernel(TrackDev tr, double t0, double dt, int32_t n_steps, float4* tab) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t total = 5 * (int64_t)n_steps + 1;
    if (i >= total) return;
    int64_t n = i / 5;
    int s = (int)(i % 5);
    const double cs[5] = {0.0, SS_C2, SS_C3, SS_C4, SS_C5};
    double t = t0 + ((double)n + cs[s]) * dt;
    double c[3];
    track_eval(tr, t, c);
    float hx = (float)c[0], hy = (float)c[1], hz = (float)c[2];
    tab[2 * i] = make_float4(hx, hy, hz, 0.f);
    tab[2 * i + 1] = make_float4((float)(c[0] - (double)hx), (float)(c[1] - (double)hy), (float)(c[2] - (double)hz), 0.f);
}

// The rotation (cos, sin)(omega t) and the frame-acceleration gradient at
// the same stage times as track_table_kernel, two float4 per slot.
__global__ void time_table_kernel(PotDev<float> P, double t0, double dt, int32_t n_steps, float4* tab) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t total = 5 * (int64_t)n_steps + 1;
    if (i >= total) return;
    int64_t n = i / 5;
    int s = (int)(i % 5);
    const double cs[5] = {0.0, SS_C2, SS_C3, SS_C4, SS_C5};
    const TimeDep<double> td = time_dep(P, t0 + ((double)n + cs[s]) * dt);
    tab[2 * i] = make_float4((float)td.c, (float)td.s, (float)td.ga[0], (float)td.ga[1]);
    tab[2 * i + 1] = make_float4((float)td.ga[2], (float)td.amp, 0.f, 0.f);
}

static bool has_time_dep(const ss_potential* pot) {
    for (int k = 0; k < pot->n_components && k < SS_MAX_COMPONENTS; ++k) {
        const int kd = pot->comp[k].kind;
        if (kd == SS_BAR || kd == SS_DEHNEN_BAR || kd == SS_UNIFORM_ACCEL || (pot->comp[k].center & SS_GROWS))
            return true;
    }
    return false;
}

// Subhalo lines relative to the run start t0: position at t0, velocity,
// (t0_s - t0, window).
__global__ void subhalo_table_kernel(ShDev sh, double t0, float4* tab) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= sh.n) return;
    double tau = t0 - sh.t0[j];
    tab[3 * j] = make_float4((float)(sh.x0[3 * j] + sh.v[3 * j] * tau), (float)(sh.x0[3 * j + 1] + sh.v[3 * j + 1] * tau),
                             (float)(sh.x0[3 * j + 2] + sh.v[3 * j + 2] * tau), (float)(sh.G * sh.m[j]));
    tab[3 * j + 1] = make_float4((float)sh.v[3 * j], (float)sh.v[3 * j + 1], (float)sh.v[3 * j + 2], (float)sh.a[j]);
    float win = isinf(sh.t_window) ? __int_as_float(0x7f800000) : (float)sh.t_window;
    tab[3 * j + 2] = make_float4((float)(sh.t0[j] - t0), win, 0.f, 0.f);
}

static int check_stream_cfg(const ss_stream_cfg* cfg, const ss_potential* pot) {
    SS_CHECK_ARG(cfg != nullptr, "cfg is NULL");
    SS_CHECK_ARG(cfg->n_particles >= 0, "n_particles < 0");
    SS_CHECK_ARG(cfg->n_steps >= 0 && cfg->n_steps < (1LL << 30), "n_steps outside [0, 2^30)");
    SS_CHECK_ARG(cfg->particles_per_release >= 1 && cfg->steps_per_release >= 0, "bad release layout");
    SS_CHECK_ARG(std::isfinite(cfg->dt) && cfg->dt > 0.0 && std::isfinite(cfg->t0), "dt must be finite and > 0");
    SS_CHECK_ARG(cfg->snap_stride >= 0, "snap_stride < 0");
    SS_CHECK_ARG(cfg->first_particle >= 0 && cfg->snap_pitch >= 0, "first_particle and snap_pitch must be >= 0");
    SS_CHECK_ARG(cfg->snap_pitch == 0 || cfg->snap_pitch >= cfg->first_particle + cfg->n_particles,
                 "snap_pitch must cover first_particle + n_particles");
    SS_CHECK_ARG(cfg->stream_particles >= 0 && cfg->subhalos_per_stream >= 0,
                 "stream_particles and subhalos_per_stream must be >= 0");
    SS_CHECK_ARG(cfg->subhalos_per_stream == 0 || cfg->stream_particles > 0,
                 "subhalos_per_stream needs stream_particles > 0");
    const int64_t end = cfg->first_particle + cfg->n_particles;
    const int64_t per_stream = cfg->stream_particles > 0 && cfg->stream_particles < end ? cfg->stream_particles : end;
    int64_t n_rel = (per_stream + cfg->particles_per_release - 1) / cfg->particles_per_release;
    SS_CHECK_ARG(n_rel == 0 || (n_rel - 1) * (int64_t)cfg->steps_per_release <= cfg->n_steps,
                 "last release starts after n_steps");
    if (cfg->subhalos_per_stream > 0) {
        const int64_t n_streams = (end + cfg->stream_particles - 1) / cfg->stream_particles;
        SS_CHECK_ARG(pot != nullptr && pot->subhalos.n >= n_streams * (int64_t)cfg->subhalos_per_stream,
                     "the subhalo table needs subhalos_per_stream rows for each of the %lld streams",
                     (long long)n_streams);
    }
    return SS_OK;
}

static StreamArgs make_args(const ss_stream_cfg* cfg, const double* ics, double* final_w, float* snaps,
                            int32_t* status) {
    StreamArgs a;
    memset(&a, 0, sizeof(a));
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
    a.grp = cfg->stream_particles;
    a.sh_per_grp = cfg->subhalos_per_stream;
    return a;
}

static bool has_expansion(const ss_potential* pot) {
    for (int k = 0; k < pot->n_components && k < SS_MAX_COMPONENTS; ++k)
        if (pot->comp[k].kind == SS_SH_EXPANSION) return true;
    return false;
}

static int64_t expansion_table_bytes(const ss_expansion& e) {
    const int64_t nt = (int64_t)(e.l_max + 1) * (e.l_max + 1);
    return (int64_t)(e.n_knots - 1) * nt * (int64_t)sizeof(float4);
}

// FP32 per-interval copy of the expansion's spline table:
// {f_k, du f'_k, f_k+1, du f'_k+1} for interval k and term j.
__global__ void expansion_table_kernel(ExpDev E, float4* out) {
    const int nt = (E.lmax + 1) * (E.lmax + 1);
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)(E.nk - 1) * nt) return;
    const int64_t k = i / nt, j = i - k * nt;
    const double* a = E.tab64 + (k * nt + j) * 2;
    const double* b = a + 2 * nt;
    out[i] = make_float4((float)a[0], (float)(a[1] * E.du), (float)b[0], (float)(b[1] * E.du));
}

int64_t expansion_table32_bytes(const ss_potential* pot) {
    return has_expansion(pot) ? expansion_table_bytes(pot->expansion) : 0;
}

int expansion_table32(PotDev<float>& P, void* ws, cudaStream_t s) {
    if (!P.ex.tab64) return SS_OK;
    float4* tab = (float4*)ws;
    const int64_t total = (int64_t)(P.ex.nk - 1) * (P.ex.lmax + 1) * (P.ex.lmax + 1);
    expansion_table_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(P.ex, tab);
    SS_LAUNCH_CHECK();
    P.ex.tab32 = tab;
    return SS_OK;
}

static int64_t f32k_workspace(const ss_potential* pot, const ss_stream_cfg* cfg) {
    int64_t bytes = 0;
    bool track = false;
    for (int k = 0; k < pot->n_components && k < SS_MAX_COMPONENTS; ++k) track |= (pot->comp[k].center & SS_CENTER_TRACK) != 0;
    if (track) bytes += (5 * cfg->n_steps + 1) * 2 * (int64_t)sizeof(float4);
    bytes = (bytes + 255) / 256 * 256;
    if (has_time_dep(pot)) bytes += (5 * cfg->n_steps + 1) * 2 * (int64_t)sizeof(float4);
    bytes = (bytes + 255) / 256 * 256;
    if (pot->subhalos.n > 0) bytes += 3 * pot->subhalos.n * (int64_t)sizeof(float4);
    bytes = (bytes + 255) / 256 * 256;
    if (has_expansion(pot)) bytes += expansion_table_bytes(pot->expansion);
    return bytes;
}

}  // namespace ssg

using namespace ssg;

extern "C" {

int ss_stream_f64(const ss_potential* pot, const ss_stream_cfg* cfg, const double* ics, double* final_w, float* snaps,
                  int32_t* status, void* stream) {
    PotDev<double> P;
    int rc = prepare_potential<double>(pot, &P, true);
    if (rc) return rc;
    rc = check_stream_cfg(cfg, pot);
    if (rc) return rc;
    if (cfg->n_particles == 0) return SS_OK;
    SS_CHECK_ARG(ics != nullptr, "ics is NULL");
    StreamArgs a = make_args(cfg, ics, final_w, snaps, status);
    const int block = F64_BLOCK;
    unsigned grid = (unsigned)((cfg->n_particles + block - 1) / block);
    // fewer warps than schedulers (4 per SM): the component-split form
    int dev = 0, sms = 0;
    SS_CUDA_TRY(cudaGetDevice(&dev));
    SS_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const bool small = P.sh.n == 0 && (cfg->n_particles + 31) / 32 < 4 * (int64_t)sms;
    dispatch_comp(P, [&](auto comp) {
        using C = decltype(comp);
        if constexpr (!std::is_same<C, GenericComp>::value) {
            if constexpr (C::n >= 3) {
                if (small) {
                    const unsigned g = (unsigned)((cfg->n_particles + 31) / 32);
                    stream_f64_split_kernel<C><<<g, 32 * C::n, 0, (cudaStream_t)stream>>>(P, a);
                    return 0;
                }
            }
        }
        stream_f64_kernel<C><<<grid, block, 0, (cudaStream_t)stream>>>(P, a);
        return 0;
    });
    SS_LAUNCH_CHECK();
    return SS_OK;
}

int64_t ss_stream_workspace_bytes(const ss_potential* pot, const ss_stream_cfg* cfg) {
    if (!pot || !cfg) return set_error(SS_ERR_INVALID_ARGUMENT, "NULL argument");
    return f32k_workspace(pot, cfg);
}

int ss_stream_f32k(const ss_potential* pot, const ss_stream_cfg* cfg, const double* ics, double* final_w,
                   float* snaps, int32_t* status, void* workspace, int64_t workspace_bytes, void* stream) {
    PotDev<float> P;
    int rc = prepare_potential<float>(pot, &P, true);
    if (rc) return rc;
    rc = check_stream_cfg(cfg, pot);
    if (rc) return rc;
    if (cfg->n_particles == 0) return SS_OK;
    SS_CHECK_ARG(ics != nullptr, "ics is NULL");
    int64_t need = f32k_workspace(pot, cfg);
    if (need > 0 && (workspace == nullptr || workspace_bytes < need))
        return set_error(SS_ERR_WORKSPACE, "workspace of %lld bytes needed, %lld given", (long long)need,
                         (long long)workspace_bytes);
    SS_CHECK_ARG(need == 0 || ((uintptr_t)workspace % 256) == 0, "workspace must be 256-byte aligned");
    cudaStream_t s = (cudaStream_t)stream;
    StreamArgs a = make_args(cfg, ics, final_w, snaps, status);
    char* ws = (char*)workspace;
    if (P.has_track) {
        float4* tab = (float4*)ws;
        int64_t total = 5 * cfg->n_steps + 1;
        track_table_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(P.track, cfg->t0, cfg->dt,
                                                                            (int32_t)cfg->n_steps, tab);
        SS_LAUNCH_CHECK();
        a.ctab = tab;
        ws += (total * 2 * (int64_t)sizeof(float4) + 255) / 256 * 256;
    }
    if (has_time_dep(pot)) {
        float4* tab = (float4*)ws;
        int64_t total = 5 * cfg->n_steps + 1;
        time_table_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(P, cfg->t0, cfg->dt, (int32_t)cfg->n_steps,
                                                                           tab);
        SS_LAUNCH_CHECK();
        a.ttab = tab;
        ws += (total * 2 * (int64_t)sizeof(float4) + 255) / 256 * 256;
    }
    if (pot->subhalos.n > 0) {
        PotDev<double> Pd;
        rc = prepare_potential<double>(pot, &Pd, true);
        if (rc) return rc;
        float4* tab = (float4*)ws;
        subhalo_table_kernel<<<(unsigned)((Pd.sh.n + 127) / 128), 128, 0, s>>>(Pd.sh, cfg->t0, tab);
        SS_LAUNCH_CHECK();
        a.shtab = tab;
        a.n_sh = Pd.sh.n;
        a.sh_kind = Pd.sh.kind;
        a.shg = Pd.sh;
        ws += (3 * Pd.sh.n * (int64_t)sizeof(float4) + 255) / 256 * 256;
    }
    if (P.ex.tab64) {
        float4* tab = (float4*)ws;
        const int64_t total = (int64_t)(P.ex.nk - 1) * (P.ex.lmax + 1) * (P.ex.lmax + 1);
        expansion_table_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(P.ex, tab);
        SS_LAUNCH_CHECK();
        P.ex.tab32 = tab;
    }
    const int block = 128;
    unsigned grid = (unsigned)((cfg->n_particles + block - 1) / block);
    if (a.n_sh > 0 && a.sh_kind == SS_SH_GRID) {
        // tabulated subhalos: one generic instantiation
        stream_f32k_kernel<GenericComp, SUB_GRID><<<grid, block, 0, s>>>(P, a);
    } else {
        dispatch_comp(P, [&](auto comp) {
            using CC = decltype(comp);
            if (a.n_sh > 0) {
                if constexpr (PairComp<CC>::ok) {
                    // two particles per thread when a pair never straddles
                    // two streams with different subhalo rows
                    if (a.sh_per_grp == 0 || (a.grp % 2 == 0 && a.p_off % 2 == 0)) {
                        const unsigned grid2 = (unsigned)(((cfg->n_particles + 1) / 2 + block - 1) / block);
                        launch_f32k2_lines<CC>(P, a, grid2, block, s);
                        return 0;
                    }
                }
                stream_f32k_kernel<CC, SUB_LINES><<<grid, block, 0, s>>>(P, a);
            } else if constexpr (PairComp<CC>::ok) {
                // two particles per thread in packed f32x2 lanes
                const unsigned grid2 = (unsigned)(((cfg->n_particles + 1) / 2 + block - 1) / block);
                stream_f32k2_kernel<CC><<<grid2, block, 0, s>>>(P, a);
            } else {
                stream_f32k_kernel<CC, SUB_NONE><<<grid, block, 0, s>>>(P, a);
            }
            return 0;
        });
    }
    SS_LAUNCH_CHECK();
    return SS_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// No-allocation variant of ss_stream_f32k.
//
// Some callers cannot allocate device memory at all: language bindings that
// reach this library through a bare C FFI and hold no device allocator, host
// code that must not make a call that may synchronize the device (cudaMalloc
// and cudaFree can), and applications whose device memory is owned entirely
// by another allocator.  For them the FP32 stream's scratch (the progenitor
// track and subhalo tables) lives in this fixed file-scope array instead of
// a caller workspace.  Every GPU that loads the library holds the array until
// the process exits.
#define SS_NOALLOC_SCRATCH_BYTES (4LL << 20)

static __device__ __align__(256) unsigned char g_noalloc_scratch[SS_NOALLOC_SCRATCH_BYTES];

#include <mutex>

namespace {
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[64] = {nullptr};
}  // namespace

// Device address of g_noalloc_scratch on the current device, looked up once
// per device (host code cannot use the symbol's host-side name as a device
// pointer) and kept for the life of the process: a cudaDeviceReset() of that
// device would leave it stale, so the entry point is not for use after one.
static int noalloc_scratch(void** out) {
    int dev = 0;
    SS_CUDA_TRY(cudaGetDevice(&dev));
    SS_CHECK_ARG(dev >= 0 && dev < 64, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (g_noalloc_ptr[dev] == nullptr) {
        void* p = nullptr;
        SS_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_noalloc_ptr[dev] = p;
    }
    *out = g_noalloc_ptr[dev];
    return SS_OK;
}

extern "C" int ss_stream_f32k_noalloc(const ss_potential* pot, const ss_stream_cfg* cfg, const double* ics,
                                      double* final_w, float* snaps, int32_t* status, void* stream) {
    if (!pot || !cfg) return set_error(SS_ERR_INVALID_ARGUMENT, "NULL argument");
    const int64_t need = f32k_workspace(pot, cfg);
    if (need > SS_NOALLOC_SCRATCH_BYTES)
        return set_error(SS_ERR_WORKSPACE,
                         "ss_stream_f32k_noalloc: this run needs %lld bytes of scratch (ss_stream_workspace_bytes) "
                         "but the fixed scratch holds %lld; use ss_stream_f32k with a workspace",
                         (long long)need, (long long)SS_NOALLOC_SCRATCH_BYTES);
    void* scratch = nullptr;
    int rc = noalloc_scratch(&scratch);
    if (rc) return rc;
    return ss_stream_f32k(pot, cfg, ics, final_w, snaps, status, scratch, SS_NOALLOC_SCRATCH_BYTES, stream);
}
