// k_front_fast_1024.cu - the specialised front-end kernel (front_fast.cuh) for
// FFT size 1024: lanes of 512 (spc 2) or 1024 (spc 1).
#include "front_fast.cuh"

namespace rd {

bool launch_front_fast_1024(const FrontParams& p, cudaStream_t s) {
  return p.spc == 2 ? dispatch_t<9, 2>(p, s) : dispatch_t<10, 1>(p, s);
}

}  // namespace rd
