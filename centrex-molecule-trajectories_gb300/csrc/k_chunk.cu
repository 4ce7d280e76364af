// libctraj.so: the chunked lens kernel (k_lens_chunk, kernels.cuh) in every
// configuration the runs and sweeps use.  Compiled on its own so that the
// kernel families build in parallel.
#include "engine.h"
#include "kernels.cuh"

namespace ctraj {
namespace {

template <bool kOut, bool kStaged, bool kRing>
LensKernel lens_kernel32(int force) {
  using M = Mol32<kOut, false>;
  switch (force) {
    case kForceStark2: return k_lens_chunk<M, kOut, kForceStark2, false, kStaged, false, kRing>;
    case kForceStark2Lin: return k_lens_chunk<M, kOut, kForceStark2Lin, false, kStaged, false, kRing>;
    case kForceStark1: return k_lens_chunk<M, kOut, kForceStark1, false, kStaged, false, kRing>;
    default: return k_lens_chunk<M, kOut, kForceRadial, false, kStaged, false, kRing>;
  }
}

template <bool kOut, bool kRing>
LensKernel lens_kernel32(int force, bool staged) {
  return staged ? lens_kernel32<kOut, true, kRing>(force) : lens_kernel32<kOut, false, kRing>(force);
}

}  // namespace

LensKernel lens_kernel(bool k64, bool out, bool ring, int force, bool staged) {
  if (k64) return out ? k_lens_chunk<Mol64<false>, true, 0, true, false> : k_lens_chunk<Mol64<false>, false, 0, true, false>;
  if (ring) return out ? lens_kernel32<true, true>(force, staged) : lens_kernel32<false, true>(force, staged);
  return out ? lens_kernel32<true, false>(force, staged) : lens_kernel32<false, false>(force, staged);
}

LensKernel sweep_lens_kernel(int force, bool staged) {
  using M = Mol32<false, false>;
  if (force == kForceStark2Lin)
    return staged ? k_lens_chunk<M, false, kForceStark2Lin, false, true, true>
                  : k_lens_chunk<M, false, kForceStark2Lin, false, false, true>;
  if (staged)
    return force == kForceStark1 ? k_lens_chunk<M, false, kForceStark1, false, true, true>
                                 : k_lens_chunk<M, false, kForceStark2, false, true, true>;
  return force == kForceStark1 ? k_lens_chunk<M, false, kForceStark1, false, false, true>
                               : k_lens_chunk<M, false, kForceStark2, false, false, true>;
}

}  // namespace ctraj
