// libctraj.so: the ballistic front kernel (k_front, kernels.cuh) in the
// configurations the runs use, and its launcher.  Compiled on its own so that
// the kernel families build in parallel.
#include "engine.h"
#include "kernels.cuh"

namespace ctraj {
namespace {

template <class M, bool kOut, int kMode>
int launch_front_t(const Plan& P, const RunDev& R, const Queue& Q, int64_t n, int threads, int sms, int waves,
                   cudaStream_t s) {
  auto kf = k_front<M, kOut, kMode>;
  const size_t smem = front_smem<M>(threads);
  CT_CUDA(cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  const int bps = blocks_per_sm(kf, threads, smem);
  const int64_t want = (n + threads - 1) / threads;
  const int grid = int(std::min<int64_t>(want, int64_t(bps) * sms * waves));
  kf<<<grid, threads, smem, s>>>(P, R, Q);
  CT_CUDA(cudaGetLastError());
  return CTRAJ_OK;
}

}  // namespace

int launch_front(const Plan& P, const RunDev& R, const Queue& Q, int64_t n, int precision, bool out, int mode,
                 int threads, int sms, int waves, cudaStream_t s) {
  using M32 = Mol32<false, false>;
  using M32o = Mol32<true, false>;
  if (precision == 64) {
    if (mode != kModePlain) return fail(CTRAJ_EINVAL, "internal error: FP64 front in mode %d", mode);
    return out ? launch_front_t<Mol64<false>, true, kModePlain>(P, R, Q, n, threads, sms, waves, s)
               : launch_front_t<Mol64<false>, false, kModePlain>(P, R, Q, n, threads, sms, waves, s);
  }
  switch (mode) {
    case kModeRing:
      return out ? launch_front_t<M32o, true, kModeRing>(P, R, Q, n, threads, sms, waves, s)
                 : launch_front_t<M32, false, kModeRing>(P, R, Q, n, threads, sms, waves, s);
    case kModeBatch:  // grouped batches have no per-molecule outputs
      if (out) return fail(CTRAJ_EINVAL, "internal error: batch front with outputs");
      return launch_front_t<M32, false, kModeBatch>(P, R, Q, n, threads, sms, waves, s);
    default:
      return out ? launch_front_t<M32o, true, kModePlain>(P, R, Q, n, threads, sms, waves, s)
                 : launch_front_t<M32, false, kModePlain>(P, R, Q, n, threads, sms, waves, s);
  }
}

}  // namespace ctraj
