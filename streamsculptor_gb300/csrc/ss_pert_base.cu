// ss_pert_base.cu — phase 1 of the subhalo response (ss_pert.cu has the
// method): one thread per particle integrates the base track in FP64 with
// the Dopri5 steps of the response and writes, per step, the six stage
// positions and tidal tensors (and, for the second order, the third
// derivatives).  First-order runs of a compiled composition (Comp<...>)
// evaluate the force and Hessian as straight-line code; the others take the
// generic component loop.  A translation unit of its own so that it
// compiles in parallel with the response kernels.

#include <cuda_runtime.h>

#include <type_traits>

#include "ss_common.cuh"
#include "ss_pert.cuh"

namespace ssg {

template <class C, class R, int ORD>
__global__ void __launch_bounds__(64) pert_base_kernel(PotDev<double> P, PertArgs a) {
    constexpr int RL = rec_len(ORD), SL = stage_len(ORD);
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.np) return;
    const int64_t p = a.p0 + i;
    const int start = (int)pert_start(p, a.ppr, a.spr);
    R* rec = reinterpret_cast<R*>(a.table) +
             (pert_offset(p, a.ppr, a.spr, a.n_steps) - pert_offset(a.p0, a.ppr, a.spr, a.n_steps)) * RL;
    double y[6];
    for (int k = 0; k < 6; ++k) y[k] = a.base_ics[6 * p + k];
    const double h = a.dt;
    const double cs[6] = {0.0, SS_C2, SS_C3, SS_C4, SS_C5, 1.0};
    for (int n = start; n < a.n_steps; ++n, rec += RL) {
        const double t = a.t0 + (double)n * h;
        double k[6][6];
        double ys[6];
#pragma unroll
        for (int s = 0; s < 6; ++s) {
            // stage state
#pragma unroll
            for (int c = 0; c < 6; ++c) {
                double acc = 0.0;
                if (s == 1) acc = SS_A21 * k[0][c];
                if (s == 2) acc = SS_A31 * k[0][c] + SS_A32 * k[1][c];
                if (s == 3) acc = SS_A41 * k[0][c] + SS_A42 * k[1][c] + SS_A43 * k[2][c];
                if (s == 4) acc = SS_A51 * k[0][c] + SS_A52 * k[1][c] + SS_A53 * k[2][c] + SS_A54 * k[3][c];
                if (s == 5)
                    acc = SS_A61 * k[0][c] + SS_A62 * k[1][c] + SS_A63 * k[2][c] + SS_A64 * k[3][c] + SS_A65 * k[4][c];
                ys[c] = s == 0 ? y[c] : y[c] + h * acc;
            }
            double g[3], r[19];
            base_stage<C, ORD>(P, ys, t + cs[s] * h, g, r);
            k[s][0] = ys[3];
            k[s][1] = ys[4];
            k[s][2] = ys[5];
            k[s][3] = -g[0];
            k[s][4] = -g[1];
            k[s][5] = -g[2];
            R* o = rec + SL * s;
#pragma unroll
            for (int c = 0; c < SL; ++c) o[c] = (R)r[c];
        }
#pragma unroll
        for (int c = 0; c < 6; ++c)
            y[c] = y[c] + h * (SS_B1 * k[0][c] + SS_B3 * k[2][c] + SS_B4 * k[3][c] + SS_B5 * k[4][c] + SS_B6 * k[5][c]);
    }
    if (a.base_out)
        for (int c = 0; c < 6; ++c) a.base_out[6 * p + c] = y[c];
}


template <class R>
static void launch_base_r(const PotDev<double>& P, const PertArgs& a, unsigned g1, cudaStream_t st) {
    if (a.ncol == 18) {
        pert_base_kernel<GenericComp, R, 2><<<g1, 64, 0, st>>>(P, a);
        return;
    }
    dispatch_comp(P, [&](auto comp) {
        using C = decltype(comp);
        pert_base_kernel<C, R, 1><<<g1, 64, 0, st>>>(P, a);
    });
}

void launch_base(const PotDev<double>& P, const PertArgs& a, int precision, unsigned g1, cudaStream_t st) {
    if (precision == 64) launch_base_r<double>(P, a, g1, st);
    else launch_base_r<float>(P, a, g1, st);
}

}  // namespace ssg
