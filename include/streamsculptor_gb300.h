/*
 * streamsculptor_gb300 — C ABI of the GB300 (sm_103a) stream-generation library.
 *
 * Everything here is plain C: pointers, sizes and POD structs.  Device
 * buffers are owned by the caller (any allocator: torch, cudaMalloc, a pool);
 * the library never allocates after the first call on a device.  Every entry
 * point is stream-ordered on the `stream` argument (a cudaStream_t passed as
 * void*; NULL = legacy default stream) and returns SS_OK (0) or a negative
 * ss_status code; ss_last_error() then gives a one-line reason (thread-local).
 *
 * Units are the reference's: kpc, Myr, Msun (G = 4.498502151469553e-12
 * kpc^3 Msun^-1 Myr^-2 is passed in ss_potential.G, so dimensionless runs work
 * too).  Each entry point names the reference interface it replaces
 * (paths relative to the jnibauer/streamsculptor source tree).
 */
#ifndef STREAMSCULPTOR_GB300_H
#define STREAMSCULPTOR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SS_ABI_VERSION 8
#define SS_MAX_COMPONENTS 16

/* ---------------------------------------------------------------- status */
typedef enum ss_status {
    SS_OK = 0,
    SS_ERR_INVALID_ARGUMENT = -1, /* null pointer, bad size, unsupported kind */
    SS_ERR_CUDA = -2,             /* a CUDA runtime call failed */
    SS_ERR_NONFINITE = -3,        /* integration produced inf/nan (per-item status set) */
    SS_ERR_WORKSPACE = -4,        /* caller workspace too small */
    SS_ERR_UNSUPPORTED = -5       /* valid request outside what this library implements */
} ss_status;

/* ------------------------------------------------------ potential model */
/* Component kinds and their raw parameters p[] (reference potential.py):
 *   SS_NFW            p = {m, r_s, soft}           NFWPotential          potential.py:74-84
 *                     (soft is added to r^2; 0 = the reference's current form)
 *   SS_TRIAXIAL_NFW   p = {m, r_s, q1, q2, q3}     TriaxialNFWPotential  potential.py:86-97
 *   SS_MIYAMOTO_NAGAI p = {m, a, b}                MiyamotoNagaiDisk     potential.py:66-72
 *   SS_HERNQUIST      p = {m, r_s, soft}           HernquistPotential    potential.py:132-138
 *   SS_PLUMMER        p = {m, r_s}                 PlummerPotential      potential.py:124-130
 *   SS_ISOCHRONE      p = {m, a}                   Isochrone             potential.py:114-122
 *   SS_SH_EXPANSION   p = {scale}                  the potential's ss_expansion table times scale
 *                     (a multipole expansion in place of the reference's optional bfeax
 *                     package; at most one expansion per potential)
 *   SS_BAR            p = {m, a, b, c, Omega}      BarPotential (Long & Murali 1992), rotating
 *                                                  about z at Omega           potential.py:178-198
 *   SS_DEHNEN_BAR     p = {alpha, v0, R0, Rb, phib, Omega}  DehnenBarPotential  potential.py:200-222
 *                     (the rotating components of one potential share one Omega)
 *   SS_UNIFORM_ACCEL  p = {}                       UniformAcceleration: gradient dv/dt of the
 *                     potential's frame_velocity track, no potential value (0)  potential.py:480-502
 *   SS_POWERLAW_CUTOFF p = {m, alpha, r_c}         PowerLawCutoffPotential (alpha < 3; the
 *                     potential value needs alpha < 2, else NaN as in the reference)
 *                                                  potential.py:357-388
 *   SS_ZHAO           p = {m, r_s, alpha, beta, gamma}  ZhaoPotential (alpha > 0, beta > 3,
 *                     0 <= gamma < 2): the gradient is dPhi/dr = G m I_z(alpha (3 - gamma),
 *                     alpha (beta - 3)) / r^2 at r + dr / 2, dr = 1e-5 r + 1e-8, which is the
 *                     reference's forward difference of Phi over [r, r + dr] to O(dr^2)
 *                                                  potential.py:282-355
 * A component with center = SS_CENTER_TRACK is evaluated at x - c(t), where
 * c(t) is the potential's center track: TimeDepTranslatingPotential,
 * potential.py:448-462.  Components are summed in list order
 * (Potential_Combine, potential.py:1279-1296). */
typedef enum ss_kind {
    SS_NFW = 1,
    SS_TRIAXIAL_NFW = 2,
    SS_MIYAMOTO_NAGAI = 3,
    SS_HERNQUIST = 4,
    SS_PLUMMER = 5,
    SS_ISOCHRONE = 6,
    SS_SH_EXPANSION = 7,
    SS_BAR = 8,
    SS_DEHNEN_BAR = 9,
    SS_UNIFORM_ACCEL = 10,
    SS_POWERLAW_CUTOFF = 11,
    SS_ZHAO = 12
} ss_kind;

/* Largest degree of a spherical-harmonic expansion. */
#define SS_SHEXP_LMAX 8

/* ss_component.center: SS_CENTER_ORIGIN or SS_CENTER_TRACK, optionally OR
 * SS_GROWS: the component is multiplied by the potential's growth track g(t)
 * (column 0 of ss_potential.growth): GrowingPotential, potential.py:464-477. */
enum { SS_CENTER_ORIGIN = 0, SS_CENTER_TRACK = 1, SS_GROWS = 4 };

typedef struct ss_component {
    int32_t kind;   /* ss_kind */
    int32_t center; /* SS_CENTER_ORIGIN or SS_CENTER_TRACK */
    double p[6];
} ss_component;

/* Center track: C1 cubic Hermite spline through knots at t0 + k*dt, with knot
 * slopes (dx/dt).  ss_track_slopes() fills the slopes the way the reference's
 * interpax.Interpolator1D(method='cubic') does (streamhelpers.py:520):
 * mean of the adjacent secants, one-sided at the two ends.  Outside
 * [t0, t0+(n-1)dt] the end cubic is extrapolated.  Pointers are device
 * pointers for device entry points. */
typedef struct ss_track {
    const double* knots;  /* [n_knots, 3] */
    const double* slopes; /* [n_knots, 3] (unused when linear) */
    double t0;
    double dt;            /* knot spacing, > 0 */
    int64_t n_knots;      /* >= 2 when any component uses the track */
    int32_t linear;       /* 1: piecewise-linear through the knots, the end
                           * segments continued (RegularGridInterpolator(method=
                           * 'linear', fill_value=None), potential.py:575-590) */
    int32_t reserved;
} ss_track;

/* Subhalos moving on straight lines x0 + v (t - t0), active while
 * |t - t0| < t_window: SubhaloLinePotential, potential.py:802-850, and its
 * d/d(r_s) companion SubhaloLinePotential_dRadius, potential.py:852-904. */
typedef enum ss_subhalo_kind { SS_SH_PLUMMER = 1, SS_SH_HERNQUIST = 2, SS_SH_GRID = 3 } ss_subhalo_kind;

typedef struct ss_subhalos {
    int32_t kind;       /* ss_subhalo_kind */
    int32_t reserved;
    int64_t n;          /* number of subhalos (0 = none) */
    const double* m;    /* [n] */
    const double* a;    /* [n] scale radius */
    const double* x0;   /* [n, 3] position at t0 */
    const double* v;    /* [n, 3] */
    const double* t0;   /* [n] */
    double t_window;    /* +inf = always active */
    /* SS_SH_GRID (TNFWSubhaloLinePotential, potential.py:1022-1108): each
     * subhalo's spherical potential as a cubic Hermite spline in u = ln r
     * through n_grid knots at grid_u0[s] + k grid_du[s], given by value and
     * d/du: grid[s][k][2]; outside the knots it continues linearly in u (the
     * reference's interpolant returns NaN there).  m and a are unused, and
     * the response to the scale radius (ncol >= 12) is not defined. */
    const double* grid;
    const double* grid_u0;
    const double* grid_du;
    int64_t n_grid;
} ss_subhalos;

/* Real spherical-harmonic expansion with spline radial functions:
 *   Phi(x) = sum_{l<=l_max} sum_{m=-l..l} f_lm(r) Y_lm(theta, phi)
 * with Schmidt semi-normalised real harmonics
 *   Y_l0 = P_l(cos theta),
 *   Y_lm = sqrt(2 (l-m)!/(l+m)!) P_l^m(cos theta) cos(m phi)     (m > 0),
 *   Y_l,-m = sqrt(2 (l-m)!/(l+m)!) P_l^m(cos theta) sin(m phi)  (m > 0),
 * P_l^m without the Condon-Shortley phase.  Term j = l*l + l + m.  Each
 * f_lm is a cubic Hermite spline in u = ln r through n_knots knots at
 * u_k = log_r0 + k*dlog_r, given by its value and du-derivative at each
 * knot; outside the knots it continues linearly in u.  coef is a device
 * pointer [n_knots][(l_max+1)^2][2] (value, d/du). */
typedef struct ss_expansion {
    int32_t l_max;        /* 0..SS_SHEXP_LMAX */
    int32_t n_knots;      /* >= 2 */
    double log_r0;
    double dlog_r;        /* > 0 */
    const double* coef;
} ss_expansion;

typedef struct ss_potential {
    double G;
    int32_t n_components;
    int32_t reserved;
    ss_component comp[SS_MAX_COMPONENTS];
    ss_track track;
    /* When subhalos.n > 0 their summed potential is part of this potential
     * (Potential_Combine([pot_base, pot_pert]), streamhelpers.py:89-146). */
    ss_subhalos subhalos;
    /* Table of the SS_SH_EXPANSION component (unused otherwise). */
    ss_expansion expansion;
    /* Velocity of the frame through time for SS_UNIFORM_ACCEL (its gradient
     * is d/dt of this track, a linear track's segment slopes; unused
     * otherwise): the MW's reflex motion of MW_LMC_Potential, potential.py:555-662. */
    ss_track frame_velocity;
    /* Growth factor g(t) of the SS_GROWS components: column 0 of this track
     * (cubic Hermite or linear like the center track; unused otherwise). */
    ss_track growth;
} ss_potential;

/* ------------------------------------------------------------- configs */
/* Particle p belongs to release r = p / particles_per_release and starts at
 * global step r * steps_per_release, i.e. at t0 + r*steps_per_release*dt,
 * then takes fixed Dormand-Prince 5(4) steps of size dt up to global step
 * n_steps (gen_stream_vmapped, main.py:343-368: every particle is integrated
 * from its release time ts[i] to ts[-1]). */
typedef struct ss_stream_cfg {
    double t0;
    double dt;                 /* > 0 */
    int64_t n_steps;
    int64_t n_particles;
    int32_t particles_per_release;
    int32_t steps_per_release;
    int32_t snap_stride;       /* 0 = final state only; else snapshot after every snap_stride global steps */
    int32_t reserved;
    /* Sub-range runs: the n_particles given are particles first_particle ..
     * first_particle + n_particles - 1 of a larger stream (their release
     * steps follow from those global indices); ics/final_w/status are indexed
     * from first_particle, snapshots are rows of snap_pitch particles
     * (0 = first_particle + n_particles) written at the global index.  Zero
     * for whole runs. */
    int64_t first_particle;
    int64_t snap_pitch;
    /* Ensembles of independent streams (jax.vmap of gen_stream_vmapped_with_pert
     * over subhalo parameters, examples/GD1_and_SubhaloFitting_GPU.ipynb):
     * with stream_particles > 0 the particles form consecutive streams of
     * stream_particles each, and the release layout above restarts in every
     * stream (global particle q is particle q % stream_particles of stream
     * q / stream_particles).  With subhalos_per_stream = k > 0, stream g feels
     * only the rows [g k, (g + 1) k) of the potential's subhalo table.  Zero
     * for a single stream.  The checkpoint / adjoint and surrogate paths take
     * single streams only. */
    int64_t stream_particles;
    int32_t subhalos_per_stream;
    int32_t reserved2;
} ss_stream_cfg;

typedef enum ss_release_model { SS_RELEASE_FARDAL = 0, SS_RELEASE_CHEN25 = 1 } ss_release_model;

/* Release (particle spray).  The reference draws its Gaussian numbers with
 * the JAX PRNG; here they are inputs (`normals`), so any generator can feed
 * them.  Fardal: 4 normals per draw (kr, kvphi, kz, kvz), main.py:209-280.
 * Chen25: 6 normals per draw, mapped to N(mean, cov) as mean + L z,
 * streamhelpers.py:352-432. */
typedef struct ss_release_cfg {
    int64_t n_release;
    int32_t n_draw;    /* draws per release; each draw gives a lead and a trail particle */
    int32_t model;     /* ss_release_model */
    double kvals[8];   /* Fardal k-values: kr_bar, kvphi_bar, kz_bar, kvz_bar, s_kr, s_kvphi, s_kz, s_kvz */
    double chen_mean[6];
    double chen_L[36]; /* row-major 6x6 factor with L L^T = cov */
} ss_release_cfg;

/* First-order response to subhalos (MassRadiusPerturbation_OTF,
 * fields.py:159-206).  Per particle: base state (6) and, per subhalo, ncol
 * columns: d(x,v)/d(eps) (6), when ncol >= 12 d^2(x,v)/d(eps)d(r_s) (6) and,
 * when ncol == 18, the second-order mass response (x2, v2) of
 * MassRadiusPerturbation_OTF_SecondOrder (fields.py:260-320):
 *   d(x2)/dt = v2,  d(v2)/dt = T x2 + (d2a/dx2 : x1 x1) - Hessian(Phi_s) x1,
 * the reference's equation as written (no factor 1/2 on either source). */
typedef struct ss_pert_cfg {
    double t0;
    double dt;                 /* signed: < 0 integrates backwards in time */
    int64_t n_steps;
    int64_t n_particles;
    int32_t particles_per_release;
    int32_t steps_per_release;
    int32_t ncol;              /* 6, 12 or 18 */
    int32_t save_stride;       /* 0 = final only; else save at steps 0, s, 2s, ... n_steps */
} ss_pert_cfg;

/* ------------------------------------------------------------ entry points */

/* Library / ABI identity. */
int ss_abi_version(void);
const char* ss_last_error(void);
/* sizeof of the ABI structs in this library: which = 0 ss_potential, 1 ss_stream_cfg,
 * 2 ss_release_cfg, 3 ss_pert_cfg, 4 ss_component, 5 ss_track, 6 ss_subhalos,
 * 7 ss_expansion, 8 ss_mlp. */
int64_t ss_abi_sizeof(int which);
/* Number of kernels this library has launched in the process so far. */
int64_t ss_kernel_launches(void);

/* Phi, grad Phi, Hessian at n points (device arrays; any output may be NULL).
 * t: per-point times [n] or NULL to use t_scalar.
 * Replaces Potential.potential / gradient / acceleration / jacobian_force
 * batched with jax.vmap (main.py:37-65; potential.py:1285-1296). */
int ss_potential_eval(const ss_potential* pot, const double* xyz, int64_t n,
                      const double* t, double t_scalar,
                      double* phi, double* grad, double* hess, void* stream);

/* Fixed-step Dopri5 orbits in FP64, one thread per orbit.
 * w0 [n_orbits, 6]; out [n_orbits, n_steps/save_every + 1, 6] holds the state
 * at steps 0, save_every, ...  dt may be negative (backwards integration).
 * Replaces Potential.integrate_orbit / integrate_orbit_batch_vmapped
 * (main.py:125-202) with dtmin = dtmax = dt. */
int ss_orbit_f64(const ss_potential* pot, const double* w0, int64_t n_orbits,
                 double t0, double dt, int64_t n_steps, int64_t save_every,
                 double* out, void* stream);

/* Ensembles of orbits that differ in step or perturbation, one thread per
 * orbit: orbit i starts at t0 from w0[i] and takes n_steps fixed Dopri5
 * steps of dt[i] (dt_all when dt is NULL; either sign), and with
 * subhalos_per_orbit = k > 0 feels only the rows [i k, (i + 1) k) of the
 * potential's subhalo table.  out as ss_orbit_f64.  Replaces jax.vmap of
 * integrate_orbit over orbits with their own end times (the back-integration
 * of stream patches to each impact time, GenerateImpactParams.py:179) or
 * their own subhalo (one perturbed progenitor per sample,
 * examples/GD1_and_SubhaloFitting_GPU.ipynb). */
int ss_orbit_ensemble_f64(const ss_potential* pot, const double* w0, int64_t n_orbits, double t0,
                          const double* dt, double dt_all, int64_t n_steps, int64_t save_every,
                          int32_t subhalos_per_orbit, double* out, void* stream);

/* One orbit, parallel in time (multiple shooting with Newton's method): the
 * n_steps fixed Dopri5 steps are split into slices that are integrated in
 * parallel in FP64 together with their 6x6 Jacobians, and a serial Newton
 * sweep joins them; converged when the joins move by less than tol
 * (relative).  The result is the serial fixed-step FP64 orbit up to
 * round-off at the joins, at a fraction of its latency on GB300.
 * out [n_steps/save_every + 1, 6]; workspace >=
 * ss_orbit_shoot_workspace_bytes(n_steps) bytes (8-byte aligned).  Static
 * potentials only; others run the serial ss_orbit_f64 kernel. */
int64_t ss_orbit_shoot_workspace_bytes(int64_t n_steps);
/* The number of slices S of an n_steps orbit (the converged slice starts,
 * [S + 1, 6] doubles, are the first 6 (S + 1) doubles of the workspace). */
int64_t ss_orbit_shoot_slices(int64_t n_steps);
int ss_orbit_shoot_f64(const ss_potential* pot, const double* w0, double t0, double dt,
                       int64_t n_steps, int64_t save_every, double* out,
                       void* workspace, int64_t workspace_bytes, double tol, void* stream);

/* Spline slopes for a center track: knots [n,3] -> slopes [n,3] (device). */
int ss_track_slopes(const double* knots, int64_t n_knots, double dt, double* slopes, void* stream);

/* Release model, FP64, one thread per (release, draw).
 * prog_w [n_release, 6] progenitor states, t_rel [n_release], msat [n_release],
 * normals [n_release, n_draw, 4 or 6]; ics [n_release, n_draw, 2, 6] with
 * index 0 = lead, 1 = trail; jac (nullable) [n_release, n_draw, 2, 6, 6] =
 * d(ics)/d(prog_w).  Replaces Potential.release_model + gen_stream_ics
 * (main.py:209-306), release_model_Chen25 (streamhelpers.py:352-459) and
 * BaseStreamModel.release_func_jacobian (perturbative.py:280-296). */
int ss_release_f64(const ss_potential* pot, const ss_release_cfg* cfg,
                   const double* prog_w, const double* t_rel, const double* msat,
                   const double* normals, double* ics, double* jac, void* stream);

/* Stream integration (the hot path).  ics [n_particles, 6] FP64.
 * final_w [n_particles, 6] FP64 state at global step n_steps (nullable).
 * snaps (nullable) [n_steps/snap_stride, n_particles, 6] float32: snapshot k
 * is the state after global step (k+1)*snap_stride; particles not yet
 * released then are NaN.  status (nullable) [n_particles]: 0 ok, 1 non-finite.
 * Replaces gen_stream_vmapped / gen_stream_scan (main.py:312-368),
 * gen_stream_vmapped_Chen25 (streamhelpers.py:491-543) and, with
 * pot->subhalos, gen_stream_vmapped_with_pert (streamhelpers.py:89-146);
 * snapshots replace the dense-output streams (main.py:376-430). */
int ss_stream_f64(const ss_potential* pot, const ss_stream_cfg* cfg, const double* ics,
                  double* final_w, float* snaps, int32_t* status, void* stream);

/* Same, FP32 stage arithmetic with compensated (hi+lo) position/velocity
 * accumulation; time and release bookkeeping stay FP64.  The progenitor
 * track and the subhalo lines are tabulated in FP32 at the run's stage times
 * into `workspace` (device, 256-byte aligned, >= ss_stream_workspace_bytes;
 * may be NULL when that is 0). */
int64_t ss_stream_workspace_bytes(const ss_potential* pot, const ss_stream_cfg* cfg);
int ss_stream_f32k(const ss_potential* pot, const ss_stream_cfg* cfg, const double* ics,
                   double* final_w, float* snaps, int32_t* status,
                   void* workspace, int64_t workspace_bytes, void* stream);

/* ss_stream_f32k for callers that cannot allocate device memory.  It has no
 * counterpart in the reference.  Some callers hold no device allocator or
 * must not call cudaMalloc/cudaFree (which may synchronize the device): a
 * bare C FFI binding, host code on a latency-critical path, an application
 * whose device memory belongs to another allocator.  This entry point takes
 * the same inputs and outputs as ss_stream_f32k (still caller-provided) and
 * keeps its scratch in a fixed 4 MiB device array inside the library
 * (SS_NOALLOC_SCRATCH_BYTES = 4194304), held by every GPU that loads the
 * library until the process exits.  A run is accepted when
 * ss_stream_workspace_bytes(pot, cfg) <= 4194304 and otherwise returns
 * SS_ERR_WORKSPACE.  The scratch is the sum of: a moving progenitor's track,
 * (5 n_steps + 1) x 32 bytes (about 26000 steps alone); a rotating or
 * frame-accelerated component, the same again (about 13000 steps together);
 * subhalo lines, 48 bytes each; an expansion, (n_knots - 1)(l_max + 1)^2 x 16
 * bytes; each part rounded up to 256 bytes.  The first call on a device
 * looks the array's device address up (cudaGetSymbolAddress) with that
 * device current; make that first call before any stream capture.  The
 * address is kept for the life of the process: do not call this entry point
 * again after cudaDeviceReset() on that device.  Every call overwrites the
 * whole scratch it uses before reading it, and all calls share the one
 * array: calls that overlap on the GPU (on streams with no ordering between
 * them, or from several host threads) race and must not be issued. */
int ss_stream_f32k_noalloc(const ss_potential* pot, const ss_stream_cfg* cfg, const double* ics,
                           double* final_w, float* snaps, int32_t* status, void* stream);

/* First-order subhalo response (fields.MassRadiusPerturbation_OTF.term,
 * fields.py:174-206, integrated as in
 * GenerateMassRadiusPerturbation.compute_perturbation_OTF, perturbative.py:100-135).
 *   base   : smooth potential (its subhalos must be empty)
 *   sh     : the subhalo table (device pointers)
 *   base_ics [n_particles, 6] FP64
 *   pert_ics [n_particles, sh->n, ncol] (nullable: zero initial response)
 *   base_out [n_particles, 6] FP64 final base state (nullable)
 *   pert_out [n_saves, n_particles, sh->n, ncol], n_saves = 1 when
 *            save_stride == 0 else n_steps/save_stride + 1
 *   workspace: device scratch of >= ss_pert_workspace_bytes(cfg, precision, 1) bytes.
 * precision: 64 -> pert_ics/pert_out are double*; 32 -> float* (FP32 response,
 * FP64 base track and time). */
int64_t ss_pert_workspace_bytes(const ss_pert_cfg* cfg, int precision, int64_t particles_per_chunk);
int ss_pert_response(const ss_potential* base, const ss_subhalos* sh, const ss_pert_cfg* cfg,
                     int precision, const double* base_ics, const void* pert_ics,
                     double* base_out, void* pert_out,
                     void* workspace, int64_t workspace_bytes, void* stream);

/* The same response along a stored base track, for many subhalo batches
 * (fields.MassRadiusPerturbation_Interp, fields.py:208-257, and
 * GenerateMassRadiusPerturbation.compute_perturbation_Interp,
 * perturbative.py:178-221: the base stream is computed once, each batch only
 * integrates its response).  ss_pert_base_track fills `track` (device,
 * >= ss_pert_track_bytes(cfg, precision) bytes: every particle's stage
 * positions and tidal tensors) and base_out (nullable); ss_pert_response_track
 * integrates the response of the subhalos `sh` (G: the base potential's G)
 * along it.  The results equal ss_pert_response's with the same cfg. */
int64_t ss_pert_track_bytes(const ss_pert_cfg* cfg, int precision);
int ss_pert_base_track(const ss_potential* base, const ss_pert_cfg* cfg, int precision, const double* base_ics,
                       double* base_out, void* track, int64_t track_bytes, void* stream);
int ss_pert_response_track(const ss_subhalos* sh, double G, const ss_pert_cfg* cfg, int precision,
                           const void* track, const void* pert_ics, void* pert_out, void* stream);

/* The response field at one point (fields.MassRadiusPerturbation_OTF.term,
 * fields.py:174-206, and MassRadiusPerturbation_OTF_SecondOrder.term,
 * fields.py:284-320): y = [x0v0 (6), sh->n x ncol] (device, FP64) at time t,
 * dy (device) receives d/dt of the same layout.  ncol: 6, 12 or 18. */
int ss_pert_term(const ss_potential* base, const ss_subhalos* sh, int ncol, double t, const double* y, double* dy,
                 void* stream);

/* Per-subhalo potential, gradient, dPhi/da and its gradient at n points
 * (device): phi [n, sh->n], grad [n, sh->n, 3], dphi_da [n, sh->n],
 * grad_dphi_da [n, sh->n, 3] (any may be NULL); zero outside the window.
 * Replaces potential_per_SH and jacfwd(potential_per_SH) of
 * SubhaloLinePotential / SubhaloLinePotential_dRadius (potential.py:832-904;
 * perturbative.py:40-41). */
int ss_subhalo_eval(const ss_subhalos* sh, double G, const double* xyz, int64_t n, double t,
                    double* phi, double* grad, double* dphi_da, double* grad_dphi_da, void* stream);

/* ---- gradients of a loss on the final stream (no reference counterpart in
 * code: the reference differentiates with jax.jacfwd through diffrax,
 * main.py:160, examples/tests.ipynb:2959).  Parameter slot 6 c + j is raw
 * parameter p[j] of component c; static potentials (no center track). */

/* ss_stream_f32k storing the compensated state every ckpt_stride (= 64) local
 * steps of each particle: ckpt [n_steps/64 + 1, n_particles, 12] floats. */
int ss_stream_f32k_ckpt(const ss_potential* pot, const ss_stream_cfg* cfg, const double* ics,
                        double* final_w, int32_t* status, float* ckpt, int32_t ckpt_stride,
                        void* stream);

/* Discrete adjoint of every particle's FP32 Dopri5 steps from the checkpoints:
 * lam_final [n_particles, 6] = dL/d(final states) -> lam_ic [n_particles, 6]
 * = dL/d(initial states); g_theta [6 n_comp] += dL/d(raw parameters). */
int ss_stream_adjoint_f32(const ss_potential* pot, const ss_stream_cfg* cfg, const float* ckpt,
                          int32_t ckpt_stride, const double* lam_final, double* lam_ic,
                          double* g_theta, void* stream);

/* Vector-Jacobian product of the release (ss_release_f64's map): lam_ics
 * [n_release, n_draw, 2, 6] -> g_prog [n_release, 6] += dL/d(progenitor
 * state) and g_theta [6 n_comp] += dL/d(raw parameters) through the tidal
 * radius; raw_params [n_comp, 6]. */
int ss_release_vjp(const ss_potential* pot, const ss_release_cfg* cfg, const double* prog_w,
                   const double* t_rel, const double* msat, const double* normals,
                   const double* lam_ics, const double* raw_params, double* g_prog,
                   double* g_theta, void* stream);

/* Progenitor orbit from the present-day state w0 back n_steps of dt and
 * forward again (FP64, parallel in time as ss_orbit_shoot_f64), with
 * forward-mode tangents along every raw parameter and every component of w0
 * (n_dir = 6 n_comp + 6): states [n_steps/save_every + 1, 6] and tangents
 * [n_steps/save_every + 1, n_dir, 6] on the forward leg.  workspace >=
 * ss_prog_tangents_workspace_bytes(n_steps, n_comp).  starts_back and
 * starts_fwd (optional, [S + 1, 6], S = ss_orbit_shoot_slices(n_steps)) are the
 * converged slice starts of the two legs from earlier ss_orbit_shoot_f64
 * calls on the same potential (the first 6 (S + 1) doubles of their
 * workspaces); given, the legs are not solved again. */
int64_t ss_prog_tangents_workspace_bytes(int64_t n_steps, int32_t n_comp);
int ss_prog_tangents_f64(const ss_potential* pot, const double* raw_params, const double* w0,
                         double dt, int32_t n_steps, int32_t save_every, double* states,
                         double* tangents, const double* starts_back, const double* starts_fwd,
                         void* workspace, int64_t workspace_bytes, void* stream);

/* Binned mean track (computed_binned_track, streamhelpers.py:201-228).
 * values [n, ncomp] FP64, key [n] FP64, edges [n_edges] ascending.
 * bin(i) = number of edges <= key[i] (numpy.digitize, right=False);
 * sums [n_edges-1, ncomp] and counts [n_edges-1, ncomp] accumulate the items
 * with bin == b for b in [0, n_edges-2], skipping NaN values per component
 * (nanmean).  Outputs are zeroed by the call. */
int ss_binned_sums(const double* values, const double* key, int64_t n, int32_t ncomp,
                   const double* edges, int32_t n_edges,
                   double* sums, double* counts, void* stream);

/* Peak arithmetic throughput probe used for rooflines: eight independent
 * FMA chains per thread on 8 blocks per SM.  precision 64, 32, or 2 for
 * packed FP32 pairs (fma.rn.f32x2, two FMAs per instruction: the form the
 * paired FP32 stream kernel issues); *out_flops = flops the launch executes;
 * sink: device buffer of >= 512 floats (never written in practice). */
int ss_peak_fma(int precision, int64_t iters, double* out_flops, float* sink, void* stream);

/* The FP64 special functions of the force evaluations, for verification
 * against the CUDA math library (no counterpart in the reference):
 * fn 0: reciprocal, 1: reciprocal square root, 2: ln(1 + x) (x >= 0);
 * out[i] = f(x[i]) and, when ref is not NULL, ref[i] = the CUDA math
 * library's 1.0 / x, rsqrt(x) or log1p(x).  x, out, ref: device [n]. */
int ss_math_f64(int fn, const double* x, int64_t n, double* out, double* ref, void* stream);

/* Strided copy of `rows` rows of `width_bytes` starting `offset_bytes`
 * into each row of pitch `pitch_bytes` (cudaMemcpy2DAsync, same offset and
 * pitch on both sides): moves a particle sub-range of snapshots
 * [n_snap, N, 6] between device and pinned host memory on `stream`.
 * kind: 0 device -> host, 1 host -> device, 2 device -> device (copy
 * engine); 3 device -> pinned host by a kernel (SM loads and stores: pinned
 * host memory is addressable from the device under unified addressing; dst
 * must be pinned host memory, src device memory, else SS_ERR_INVALID_ARGUMENT). */
int ss_copy_rows_async(void* dst, const void* src, int64_t rows, int64_t pitch_bytes, int64_t offset_bytes,
                       int64_t width_bytes, int kind, void* stream);

/* ---------------------------------------------------- MLP force surrogate
 * A learned potential for expensive expansion potentials:
 *   Phi(x) ~ out_scale * N(u) + out_shift,
 *   u = ((x - in_shift[0]) in_scale[0], (y - in_shift[1]) in_scale[1],
 *        (z - in_shift[2]) in_scale[2], (ln r - in_shift[3]) in_scale[3]),
 *   N: 4 -> 128 -> 128 -> 128 -> 128 -> 1 with SiLU after each hidden layer;
 * the force is the network's analytic input gradient (hand-written
 * backward).  params: device FP32, packed as
 *   W1 [128][4], b1 [128], W2 [128][128], b2 [128], W3, b3, W4, b4,
 *   w5 [128], b5 [1]   (W[out][in], SS_MLP_NPARAM floats). */
#define SS_MLP_WIDTH 128
#define SS_MLP_NPARAM (128 * 4 + 128 + 3 * (128 * 128 + 128) + 128 + 1)

typedef struct ss_mlp {
    const float* params;
    float in_scale[4];
    float in_shift[4];
    float out_scale;
    float out_shift;
    /* Optional exact spherical part Phi_0(r) added to the network (NULL =
     * none): a cubic Hermite spline in u = ln r through base_n knots at
     * base_u0 + k base_du, [base_n][2] (value, d/du) FP64 on the device,
     * continued linearly in u outside the knots (the form of an expansion's
     * l = 0 radial function).  The network then represents Phi - Phi_0 (it
     * is trained on that residual) and every evaluation adds Phi_0 and its
     * gradient exactly: FP64 in ss_mlp_eval, FP32 from a shared-memory copy
     * in the tensor-core kernels (2 <= base_n <= SS_MLP_BASE_MAX). */
    const double* base;
    int32_t base_n;
    int32_t reserved;
    double base_u0;
    double base_du;
} ss_mlp;

#define SS_MLP_BASE_MAX 256

/* FP32 evaluation (CUDA cores) of Phi and grad Phi at n points xyz [n,3]
 * (either output may be NULL).  Workspace: ss_mlp_eval_workspace_bytes(n). */
int64_t ss_mlp_eval_workspace_bytes(int64_t n);
int ss_mlp_eval(const ss_mlp* mlp, const double* xyz, int64_t n, double* phi, double* grad,
                void* workspace, int64_t workspace_bytes, void* stream);

/* Training loss of one batch and its gradient with respect to params:
 *   L = sum_b w_val[b] (Phi_b - phi_t[b])^2 + w_force[b] |grad Phi_b - g_t[b]|^2
 * (Sobolev training: the force term is differentiated through the network's
 * input gradient).  x [B,3], phi_t [B], g_t [B,3] (grad Phi targets),
 * w_val, w_force [B] FP32 device arrays.  Writes loss[0] (value part),
 * loss[1] (force part) and grad [SS_MLP_NPARAM] (overwritten).
 * Workspace: ss_mlp_train_workspace_bytes(B). */
int64_t ss_mlp_train_workspace_bytes(int64_t batch);
int ss_mlp_loss_grad(const ss_mlp* mlp, const float* x, const float* phi_t, const float* g_t,
                     const float* w_val, const float* w_force, int64_t batch, float* loss, float* grad,
                     void* workspace, int64_t workspace_bytes, void* stream);

/* The whole Adam fit, run by the library: for step s = 0 .. steps-1 the
 * batch is samples order[s*batch .. s*batch + batch - 1] of the training
 * set (x [n,3], phi_t [n], g_t [n,3], w_val, w_force [n] FP32 device
 * arrays; order int32 device [steps*batch], indices < n), its loss gradient
 * as ss_mlp_loss_grad, then one Adam step with the learning rate
 * lr_min + (lr - lr_min) (1 + cos(pi s / (steps - 1))) / 2 and the bias
 * corrections of step s + 1.  params [SS_MLP_NPARAM] (device) are updated in
 * place and take the place of mlp->params (the rest of mlp: normalisation,
 * exact base); m, v [SS_MLP_NPARAM]: the Adam moments, zero for a fresh fit.
 * loss_log (device [steps][2], nullable): each step's (value, force) loss.
 * No host synchronisation inside.  Workspace: ss_mlp_fit_workspace_bytes(batch). */
int64_t ss_mlp_fit_workspace_bytes(int64_t batch);
int ss_mlp_fit(const ss_mlp* mlp, float* params, const float* x, const float* phi_t, const float* g_t,
               const float* w_val, const float* w_force, int64_t n, const int32_t* order, int64_t batch,
               int64_t steps, float lr, float lr_min, float beta1, float beta2, float eps, float* m, float* v,
               float* loss_log, void* workspace, int64_t workspace_bytes, void* stream);

/* Which units run the training's 128-wide products (every ss_mlp_loss_grad
 * and ss_mlp_eval GEMM with N = 128 and K a multiple of 32): 1 (default) the
 * tensor cores (tcgen05 kind::tf32, each FP32 operand split into a TF32 head
 * and remainder, three MMAs per product: about 1e-5 relative, where one
 * TF32 product would give about 1e-3), 0 the CUDA-core FP32 GEMM.  Other values leave the setting.  Returns the previous setting.
 * Process-wide: set it between calls, not while a call is in flight. */
int ss_mlp_train_backend(int tensor_cores);

/* One Adam step (bias-corrected; step counts from 1) on n parameters. */
int ss_mlp_adam(float* params, const float* grad, float* m, float* v, int64_t n, int64_t step, float lr,
                float beta1, float beta2, float eps, void* stream);

/* grad Phi of the surrogate at xyz [n,3] through the tensor-core path of
 * ss_stream_mlp_bf16 (BF16 weights and activations, FP32 accumulation).
 * status [n] (optional): 0, or 2 if a tensor-core wait timed out. */
int ss_mlp_grad_bf16(const ss_mlp* mlp, const double* xyz, int64_t n, double* grad, int32_t* status,
                     void* stream);

/* Particle-spray stream with the surrogate's force on the tensor cores
 * (tcgen05, BF16 weights and activations, FP32 accumulation in TMEM), FP32
 * compensated state, FP64 time: the ss_stream_f32k contract with the force
 * of `mlp` in place of a potential.  Workspace:
 * ss_stream_mlp_workspace_bytes(cfg). */
int64_t ss_stream_mlp_workspace_bytes(const ss_stream_cfg* cfg);
int ss_stream_mlp_bf16(const ss_mlp* mlp, const ss_stream_cfg* cfg, const double* ics, double* final_w,
                       float* snaps, int32_t* status, void* workspace, int64_t workspace_bytes, void* stream);

/* The same with the exact potential kept as error judge and fallback (the
 * force it replaces is Potential.gradient, main.py:37-40): every
 * judge_every steps of each 128-particle tile (counted from the tile's
 * first step), the surrogate's force at the step's starting point is
 * compared with `exact`'s force (FP32, CUDA cores) for every particle of
 * the tile; if any |g_mlp - g_exact| > tol |g_exact| (or either is not
 * finite), the tile integrates with the exact force from that step to the
 * end of the run.  fallbacks (device int64, optional; not
 * zeroed by the call) is incremented once per tile that fell back.  exact:
 * a static potential of the analytic kinds and/or an l_max = 8 expansion
 * (no center track, subhalos or rotation).  Workspace:
 * ss_stream_mlp_judged_workspace_bytes(exact, cfg) (the expansion's FP32
 * interval table), 256-byte aligned. */
int64_t ss_stream_mlp_judged_workspace_bytes(const ss_potential* exact, const ss_stream_cfg* cfg);
int ss_stream_mlp_judged_bf16(const ss_mlp* mlp, const ss_potential* exact, const ss_stream_cfg* cfg, float tol,
                              int32_t judge_every, const double* ics, double* final_w, float* snaps,
                              int32_t* status, int64_t* fallbacks, void* workspace, int64_t workspace_bytes,
                              void* stream);

#ifdef __cplusplus
}
#endif

#endif /* STREAMSCULPTOR_GB300_H */
