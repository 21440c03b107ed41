// Fused panel-recursion node (panel_node.cuh), FP32 instantiations: the
// two precisions compile as separate translation units, in parallel.
#include "panel_node.cuh"

namespace gb {
template int panel_node_dev<float>(float*, int, int, int, int, int*, cudaStream_t);
}  // namespace gb
