// Radix argsort (placeholder registration until the kernels land).
#include "registry.h"
namespace vkc {
void register_sort(std::vector<KernelDef> &) {}
}  // namespace vkc
