// k_front_fast.cu - the specialised front-end kernel for FFT sizes 16 and 64
// (front_fast.cuh), and the dispatch over every specialised geometry.
#include "front_fast.cuh"

namespace rd {

bool launch_front_fast_small(const FrontParams& p, cudaStream_t s) {
  if (p.spc == 2) {
    if (p.N == 16) return dispatch_t<3, 2>(p, s);
    if (p.N == 64) return dispatch_t<5, 2>(p, s);
    return false;
  }
  return p.N == 64 ? dispatch_t<6, 1>(p, s) : false;
}

// Whether launch_front_fast has a specialisation for the geometry.
bool front_fast_ok(uint32_t n, uint32_t spc) {
  switch (n) {
    case 16: return spc == 2;
    case 64: return spc == 1 || spc == 2;
    case 256:
    case 1024: return spc == 1 || spc == 2;
    default: return false;
  }
}

// Launches the specialised kernel when the geometry has one; returns false
// otherwise (the caller then uses the generic k_front).
bool launch_front_fast(const FrontParams& p, cudaStream_t s) {
  switch (p.N) {
    case 16:
    case 64: return launch_front_fast_small(p, s);
    case 256: return launch_front_fast_256(p, s);
    case 1024: return launch_front_fast_1024(p, s);
    default: return false;
  }
}

}  // namespace rd
