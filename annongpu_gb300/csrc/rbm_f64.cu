// RBM-family launchers instantiated for double arithmetic.
#include "rbm_launch.cuh"

namespace ann {
template void rbm_prepare_T<double>(ann_psi_impl&, cudaStream_t);
template void rbm_mc_T<double>(ann_psi_impl&, const ann_op_impl*, ann_ens_impl&, const SampleTargets&, cudaStream_t);
template void rbm_exact_T<double>(ann_psi_impl&, const ann_op_impl*, ann_ens_impl&, const SampleTargets&, cudaStream_t);
template void rbm_confs_T<double>(ann_psi_impl&, const ann_op_impl*, const uint64_t*, size_t, Rows&, void*, size_t,
                                cudaStream_t);
}  // namespace ann
