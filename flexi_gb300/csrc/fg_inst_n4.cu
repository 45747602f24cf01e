// flexi_gb300 -- kernel instantiation for 4 nodes per direction (N = 3)
#include "fg_inst.cuh"
namespace fg {
KernelSet kernel_set_n4(bool gl) { return gl ? Inst<4, true>::make() : Inst<4, false>::make(); }
}  // namespace fg
