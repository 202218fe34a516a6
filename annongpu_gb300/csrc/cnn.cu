// PsiCNN on the GPU (include/quantum_state/PsiCNN.hpp:97-266).
#include "ann_internal.hpp"

namespace ann {

void cnn_prepare(ann_psi_impl&, cudaStream_t) { throw Error(ANN_ERR_UNSUPPORTED, "PsiCNN kernels not built yet"); }
void cnn_run(ann_psi_impl&, const ann_op_impl*, ann_ens_impl&, const SampleTargets&, cudaStream_t) {
    throw Error(ANN_ERR_UNSUPPORTED, "PsiCNN kernels not built yet");
}
void cnn_confs(ann_psi_impl&, const ann_op_impl*, const uint64_t*, size_t, Rows&, void*, size_t, cudaStream_t) {
    throw Error(ANN_ERR_UNSUPPORTED, "PsiCNN kernels not built yet");
}

}  // namespace ann

extern "C" int ann_psi_create_cnn(const ann_cnn_desc*, ann_psi**) { return ANN_ERR_UNSUPPORTED; }
