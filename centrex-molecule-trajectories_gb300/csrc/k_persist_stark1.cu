// libctraj.so: the persistent FP32 lens kernel's configurations for the
// force law kForceStark1 (see k_persist.cuh).
#include "k_persist.cuh"

namespace ctraj {
template PersistKernel persist_kernel_for<kForceStark1>(bool, int, bool, int, int, int*, int*);
}  // namespace ctraj
