// flexi_gb300 -- kernel instantiation for 2 nodes per direction (N = 1)
#include "fg_inst.cuh"
namespace fg {
KernelSet kernel_set_n2(bool gl) { return gl ? Inst<2, true>::make() : Inst<2, false>::make(); }
}  // namespace fg
