// flexi_gb300 -- kernel instantiation for 11 nodes per direction (N = 10)
#include "fg_inst.cuh"
namespace fg {
KernelSet kernel_set_n11(bool gl) { return gl ? Inst<11, true>::make() : Inst<11, false>::make(); }
}  // namespace fg
