// group_id (placeholder registration until the kernels land).
#include "registry.h"
namespace vkc {
void register_group(std::vector<KernelDef> &) {}
}  // namespace vkc
