// Instances of the third-generation FP32 column kernel for up to 4 precession
// angle(s) per pass (one translation unit per angle bucket, compiled in parallel).
#include "k_column_v3.cuh"

namespace stem {
namespace ring3 {
template cudaError_t ring3_launch_np<4>(const Ring3Args& a);
}  // namespace ring3
}  // namespace stem
