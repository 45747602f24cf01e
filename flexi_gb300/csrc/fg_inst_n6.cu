// flexi_gb300 -- kernel instantiation for 6 nodes per direction (N = 5)
#include "fg_inst.cuh"
namespace fg {
KernelSet kernel_set_n6(bool gl) { return gl ? Inst<6, true>::make() : Inst<6, false>::make(); }
}  // namespace fg
