// mc_f64.cu -- the track-loop kernels of mc_impl.cuh instantiated for double (FP64 kinematics).
#include "mc_impl.cuh"

namespace tk {

size_t shi_event_bytes() { return sizeof(ShiEv); }

template void launch_propose<double>(const Proposer&, const McConst<double>&, const DevTabs<double>&, PQ<double>,
                                     PQ<double>, const Ctrs*, cudaStream_t);
template void launch_shi<double>(const McConst<double>&, const DevShi<double>&, void*, int64_t, Ctrs*, int, cudaStream_t,
                                 int, unsigned long long*);
template void launch_pairs<double>(const McConst<double>&, const DevTabs<double>&, const void*, int64_t, PQ<double>,
                                   PQ<double>, PQ<double>, Tal, Ctrs*, cudaStream_t, const InstInfo*);
template void launch_step<double>(const McConst<double>&, const DevTabs<double>&, const QSet<double>&, const int*,
                                  const QSet<double>&, PQ<double>, PQ<double>, Tal, Ctrs*, int, int, int, cudaStream_t,
                                  const float*, const Proposer*, const Fork*);
template void launch_probe<double>(const McConst<double>&, const DevTabs<double>&, const DevShi<double>&, int, int,
                                   int, const double*, const double*, double*, cudaStream_t);
template void launch_grid_hints<double>(const McConst<double>&, GHint<double>*, GHint<double>*, cudaStream_t);

}  // namespace tk
