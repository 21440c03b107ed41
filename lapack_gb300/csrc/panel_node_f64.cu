// Fused panel-recursion node (panel_node.cuh), FP64 instantiations: the
// two precisions compile as separate translation units, in parallel.
#include "panel_node.cuh"

namespace gb {
template int panel_node_dev<double>(double*, int, int, int, int, int*, cudaStream_t);
}  // namespace gb
