// libctraj.so: the persistent FP32 lens kernel's configurations for the
// force law kForceStark2Lin (see k_persist.cuh).
#include "k_persist.cuh"

namespace ctraj {
template PersistKernel persist_kernel_for<kForceStark2Lin>(bool, int, bool, int, int, int*, int*);
}  // namespace ctraj
