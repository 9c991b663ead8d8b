// mc_f32.cu -- the track-loop kernels of mc_impl.cuh instantiated for float (FP32 kinematics).
#include "mc_impl.cuh"

namespace tk {

template void launch_propose<float>(const Proposer&, const McConst<float>&, const DevTabs<float>&, PQ<float>,
                                    PQ<float>, const Ctrs*, cudaStream_t);
template void launch_shi<float>(const McConst<float>&, const DevShi<float>&, void*, int64_t, Ctrs*, int, cudaStream_t,
                                int, unsigned long long*);
template void launch_pairs<float>(const McConst<float>&, const DevTabs<float>&, const void*, int64_t, PQ<float>,
                                  PQ<float>, PQ<float>, Tal, Ctrs*, cudaStream_t, const InstInfo*);
template void launch_step<float>(const McConst<float>&, const DevTabs<float>&, const QSet<float>&, const int*,
                                 const QSet<float>&, PQ<float>, PQ<float>, Tal, Ctrs*, int, int, int, cudaStream_t,
                                 const float*, const Proposer*, const Fork*);
template void launch_probe<float>(const McConst<float>&, const DevTabs<float>&, const DevShi<float>&, int, int, int,
                                  const double*, const double*, double*, cudaStream_t);
template void launch_grid_hints<float>(const McConst<float>&, GHint<float>*, GHint<float>*, cudaStream_t);

}  // namespace tk
