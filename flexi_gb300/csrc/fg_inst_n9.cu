// flexi_gb300 -- kernel instantiation for 9 nodes per direction (N = 8)
#include "fg_inst.cuh"
namespace fg {
KernelSet kernel_set_n9(bool gl) { return gl ? Inst<9, true>::make() : Inst<9, false>::make(); }
}  // namespace fg
