// The panel factorisations in FP32 (see tf_nd_panel.cuh).

#include "tf_nd_panel.cuh"

namespace tf {
namespace nd {

template int panel<float>(const DevPlan &, int, int, int, int, int, float *, int32_t *, int32_t *, cudaStream_t);

}  // namespace nd
}  // namespace tf
