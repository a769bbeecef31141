#include "pls.cuh"
namespace oh {
oh_status pls_tensor_enqueue(oh_ctx*, const PlsGeom&, const PlsPt*, int, void*, cudaStream_t) {
  return fail(OH_ERR_UNSUPPORTED_SIZE, "tensor engine not built");
}
}  // namespace oh
