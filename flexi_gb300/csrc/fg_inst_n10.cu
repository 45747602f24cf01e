// flexi_gb300 -- kernel instantiation for 10 nodes per direction (N = 9)
#include "fg_inst.cuh"
namespace fg {
KernelSet kernel_set_n10(bool gl) { return gl ? Inst<10, true>::make() : Inst<10, false>::make(); }
}  // namespace fg
