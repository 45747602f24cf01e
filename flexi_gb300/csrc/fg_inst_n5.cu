// flexi_gb300 -- kernel instantiation for 5 nodes per direction (N = 4)
#include "fg_inst.cuh"
namespace fg {
KernelSet kernel_set_n5(bool gl) { return gl ? Inst<5, true>::make() : Inst<5, false>::make(); }
}  // namespace fg
