// flexi_gb300 -- kernel instantiation for 3 nodes per direction (N = 2)
#include "fg_inst.cuh"
namespace fg {
KernelSet kernel_set_n3(bool gl) { return gl ? Inst<3, true>::make() : Inst<3, false>::make(); }
}  // namespace fg
