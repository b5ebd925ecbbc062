// ss_stream2.cu — the packed two-particle FP32 stream kernel with analytic
// subhalo lines (stream_f32k2_kernel<C, SUB_LINES>), one instantiation per
// compiled composition that has a packed force.  These serve the perturbed
// streams of gen_stream_vmapped_with_pert (streamhelpers.py:89-146) and the
// ensembles of perturbed streams of the subhalo-fitting notebook, whose
// subhalos are Plummer or Hernquist lines (potential.py:802-904).  Kept in a
// translation unit of its own so that it compiles in parallel with
// ss_stream.cu; ss_stream_f32k (ss_stream.cu) decides when to launch it.

#include <cuda_runtime.h>

#include "ss_stream2.cuh"

namespace ssg {

template <class C>
void launch_f32k2_lines(const PotDev<float>& P, const StreamArgs& a, unsigned grid, int block, cudaStream_t s) {
    static_assert(PairComp<C>::ok, "composition without a packed force");
    stream_f32k2_kernel<C, SUB_LINES><<<grid, block, 0, s>>>(P, a);
}

template void launch_f32k2_lines<CompMW3>(const PotDev<float>&, const StreamArgs&, unsigned, int, cudaStream_t);
template void launch_f32k2_lines<CompMW3P>(const PotDev<float>&, const StreamArgs&, unsigned, int, cudaStream_t);
template void launch_f32k2_lines<CompGala>(const PotDev<float>&, const StreamArgs&, unsigned, int, cudaStream_t);
template void launch_f32k2_lines<CompGalaP>(const PotDev<float>&, const StreamArgs&, unsigned, int, cudaStream_t);
template void launch_f32k2_lines<CompTri3>(const PotDev<float>&, const StreamArgs&, unsigned, int, cudaStream_t);
template void launch_f32k2_lines<CompTri3P>(const PotDev<float>&, const StreamArgs&, unsigned, int, cudaStream_t);
template void launch_f32k2_lines<CompNFW>(const PotDev<float>&, const StreamArgs&, unsigned, int, cudaStream_t);
template void launch_f32k2_lines<CompPlummer>(const PotDev<float>&, const StreamArgs&, unsigned, int,
                                              cudaStream_t);

}  // namespace ssg
