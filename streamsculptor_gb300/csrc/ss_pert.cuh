// ss_pert.cuh — what the two phases of the subhalo response share (the
// base-track records and the launch arguments); phase 1 (the FP64 base
// track) is in ss_pert_base.cu, phase 2 (the response) in ss_pert.cu.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "ss_device.cuh"

namespace ssg {

// Base-track records per step: first order 6 stages x (x0[3], T[6]) + 2 pad;
// second order (ncol = 18) adds the 10 independent third derivatives of the
// base acceleration per stage: 6 x 19 + 6 pad.
static constexpr int REC = 56;
static constexpr int REC2 = 120;
__host__ __device__ constexpr int rec_len(int ord) { return ord == 2 ? REC2 : REC; }
__host__ __device__ constexpr int stage_len(int ord) { return ord == 2 ? 19 : 9; }

struct PertArgs {
    int64_t N;       // particles in the whole run
    int64_t p0;      // first particle of the chunk
    int64_t np;      // particles in the chunk
    int32_t ppr;
    int32_t spr;
    int32_t n_steps;
    int32_t ncol;
    int32_t save_stride;
    int32_t n_saves;
    double t0;
    double dt;
    const double* base_ics;
    double* base_out;
    const void* pert_ics;
    void* pert_out;
    void* table;
};

__host__ __device__ inline int64_t pert_start(int64_t p, int32_t ppr, int32_t spr) { return (p / ppr) * (int64_t)spr; }

// Number of records (steps) of particles [0, p): sum of (n_steps - start_q).
__host__ __device__ inline int64_t pert_offset(int64_t p, int32_t ppr, int32_t spr, int32_t n_steps) {
    int64_t R = p / ppr;
    int64_t floors = (int64_t)ppr * (R * (R - 1) / 2) + (p - R * ppr) * R;
    return p * (int64_t)n_steps - (int64_t)spr * floors;
}

// ------------------------------------------------------------- phase 1
// One stage record of the base track at (x, t): x0, T = -Hessian(Phi)
// (xx yy zz xy xz yz) and, for the second order, d2a/dx dx = -(third
// derivatives of Phi) by forward-mode differentiation of the analytic
// Hessian, ordered xxx xxy xxz xyy xyz xzz yyy yyz yzz zzz.  g = grad Phi.
template <class C, int ORD>
__device__ __forceinline__ void base_stage(const PotDev<double>& P, const double x[3], double t, double g[3],
                                           double r[19]) {
    double cc[3] = {0.0, 0.0, 0.0};
    if (P.has_track) track_eval(P.track, t, cc);
    double H[6];
    const double xs[3] = {x[0] - cc[0], x[1] - cc[1], x[2] - cc[2]};
    const TimeDep<double> td = time_dep(P, t);
    C::template grad<double, double, true>(P, x, xs, g, H, td);
    r[0] = x[0];
    r[1] = x[1];
    r[2] = x[2];
#pragma unroll
    for (int c = 0; c < 6; ++c) r[3 + c] = -H[c];
    if constexpr (ORD == 2) {
        Dual<3> xd[3], xsd[3], gd[3], Hd[6];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            xd[c] = Dual<3>(x[c]);
            xd[c].d[c] = 1.0;
            xsd[c] = Dual<3>(xs[c]);
            xsd[c].d[c] = 1.0;
        }
        pot_grad<Dual<3>, double, true>(P, xd, xsd, gd, Hd, time_dep_as<Dual<3>>(td));
        // H order xx yy zz xy xz yz; D_abc = d H_ab / d x_c
        const double D[10] = {Hd[0].d[0], Hd[0].d[1], Hd[0].d[2], Hd[1].d[0], Hd[3].d[2],
                              Hd[2].d[0], Hd[1].d[1], Hd[1].d[2], Hd[2].d[1], Hd[2].d[2]};
#pragma unroll
        for (int c = 0; c < 10; ++c) r[9 + c] = -D[c];
    }
}

// Phase 1 over the particles [a.p0, a.p0 + a.np) (g1 blocks of 64): the
// compiled composition of P when there is one (first order), else the
// generic loop.
void launch_base(const PotDev<double>& P, const PertArgs& a, int precision, unsigned g1, cudaStream_t st);

}  // namespace ssg
