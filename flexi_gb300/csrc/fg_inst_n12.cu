// flexi_gb300 -- kernel instantiation for 12 nodes per direction (N = 11)
#include "fg_inst.cuh"
namespace fg {
KernelSet kernel_set_n12(bool gl) { return gl ? Inst<12, true>::make() : Inst<12, false>::make(); }
}  // namespace fg
