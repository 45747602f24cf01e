// flexi_gb300 -- kernel instantiation for 7 nodes per direction (N = 6)
#include "fg_inst.cuh"
namespace fg {
KernelSet kernel_set_n7(bool gl) { return gl ? Inst<7, true>::make() : Inst<7, false>::make(); }
}  // namespace fg
