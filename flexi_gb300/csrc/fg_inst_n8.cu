// flexi_gb300 -- kernel instantiation for 8 nodes per direction (N = 7)
#include "fg_inst.cuh"
namespace fg {
KernelSet kernel_set_n8(bool gl) { return gl ? Inst<8, true>::make() : Inst<8, false>::make(); }
}  // namespace fg
