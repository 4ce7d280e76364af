// The persistent FP32 lens kernel's configurations for one force law
// (persist_kernel_for<F>), explicitly instantiated by k_persist_<law>.cu so
// that the four force laws compile in parallel; k_persist.cu dispatches.
#pragma once
#include "engine.h"
#include "kernels.cuh"

namespace ctraj {

template <bool kOut, int F, bool kStaged, int kMode>
PersistKernel persist_kernel_t(int lanes, int mpt, int* threads, int* used_mpt) {
  using M = Mol32<kOut, false>;
  *used_mpt = 1;
  if constexpr (!kOut && kStaged && (kMode == kModePlain || kMode == kModeBatch)) {
    if constexpr (F == kForceStark2 || F == kForceStark2Lin) {
      if (mpt == 2) {
        *used_mpt = 2;
        *threads = lanes / 2;
        if (lanes == 1024) return k_lens_persist<M, kOut, F, kStaged, kMode, 512, 2>;
        if (lanes == 768) return k_lens_persist<M, kOut, F, kStaged, kMode, 384, 2>;
        *threads = 256;
        return k_lens_persist<M, kOut, F, kStaged, kMode, 256, 2>;
      }
    }
    if (lanes == 1024) {
      *threads = 1024;
      return k_lens_persist<M, kOut, F, kStaged, kMode, 1024>;
    }
    if (lanes == 768) {
      *threads = 768;
      return k_lens_persist<M, kOut, F, kStaged, kMode, 768>;
    }
  }
  *threads = kPersistThreads;
  return k_lens_persist<M, kOut, F, kStaged, kMode, kPersistThreads>;
}

template <bool kOut, int F, int kMode>
PersistKernel persist_kernel_m(bool staged, int lanes, int mpt, int* threads, int* used_mpt) {
  return staged ? persist_kernel_t<kOut, F, true, kMode>(lanes, mpt, threads, used_mpt)
                : persist_kernel_t<kOut, F, false, kMode>(lanes, mpt, threads, used_mpt);
}

template <int F>
PersistKernel persist_kernel_for(bool out, int mode, bool staged, int lanes, int mpt, int* threads, int* used_mpt) {
  if (mode == kModeRing)
    return out ? persist_kernel_m<true, F, kModeRing>(staged, lanes, mpt, threads, used_mpt)
               : persist_kernel_m<false, F, kModeRing>(staged, lanes, mpt, threads, used_mpt);
  if (mode == kModeBatch)  // grouped batches have no per-molecule outputs
    return persist_kernel_m<false, F, kModeBatch>(staged, lanes, mpt, threads, used_mpt);
  return out ? persist_kernel_m<true, F, kModePlain>(staged, lanes, mpt, threads, used_mpt)
             : persist_kernel_m<false, F, kModePlain>(staged, lanes, mpt, threads, used_mpt);
}

}  // namespace ctraj
