// k_front_fast_256.cu - the specialised front-end kernel (front_fast.cuh) for
// FFT size 256: lanes of 128 (spc 2) or 256 (spc 1).
#include "front_fast.cuh"

namespace rd {

bool launch_front_fast_256(const FrontParams& p, cudaStream_t s) {
  return p.spc == 2 ? dispatch_t<7, 2>(p, s) : dispatch_t<8, 1>(p, s);
}

}  // namespace rd
