// libctraj.so: the persistent FP32 lens kernel (k_lens_persist, kernels.cuh):
// the dispatch over force laws; each law's configurations are compiled in a
// translation unit of its own (k_persist_<law>.cu, from k_persist.cuh).
#include "engine.h"
#include "kernels.cuh"

namespace ctraj {

static_assert(sizeof(DoneRec) == kDoneRecBytes, "DoneRec layout");

FinishKernel finish_kernel(int mode) {
  using M = Mol32<false, false>;
  if (mode == kModeSweep) return k_lens_finish<M, kModeSweep>;
  return mode == kModeBatch ? k_lens_finish<M, kModeBatch> : k_lens_finish<M, kModePlain>;
}

PersistKernel persist_kernel(bool out, int force, int mode, bool staged, int lanes, int mpt, int* threads,
                             int* used_mpt) {
  switch (force) {
    case kForceStark2: return persist_kernel_for<kForceStark2>(out, mode, staged, lanes, mpt, threads, used_mpt);
    case kForceStark2Lin: return persist_kernel_for<kForceStark2Lin>(out, mode, staged, lanes, mpt, threads, used_mpt);
    case kForceStark1: return persist_kernel_for<kForceStark1>(out, mode, staged, lanes, mpt, threads, used_mpt);
    default: return persist_kernel_for<kForceRadial>(out, mode, staged, lanes, mpt, threads, used_mpt);
  }
}

}  // namespace ctraj
