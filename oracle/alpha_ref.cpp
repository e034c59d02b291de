// alpha_ref.cpp -- TEST INFRASTRUCTURE ONLY: a C entry point over the
// reference's own BufferedAlphaNoise (core/noise.hpp:138-241), built from
// the reference checkout by oracle/build_ref.sh into oracle/_ref/, so that
// tests/golden/make_alpha_noise.py can record the reference's buffers
// together with the white draws that produced them.  The product never
// loads it.  The un-vendored kissfft comes from the project-written
// stand-in under oracle/stubs/ (an exact DFT).
#include <cstdint>
#include <cstring>

#include "noise.hpp"

namespace {
// The reference class with a seedable generator and its white buffer in
// view (both are protected members).
struct Exposed : public BufferedAlphaNoise<double> {
  Exposed(unsigned n, double alpha, double std_, unsigned seed) : BufferedAlphaNoise<double>(n, alpha, std_, 1.0) {
    this->generator.seed(seed);
  }
  const std::complex<float> *white() const { return this->bufferWhite.data(); }
};
}  // namespace

extern "C" {
// One fillBuffer() of BufferedAlphaNoise(n, alpha, std, 1) with its
// mt19937 seeded by `seed`: white[0..n) are the draws, out[0..n) the buffer.
int alpha_ref_fill(uint32_t n, double alpha, double std_, uint32_t seed, float *white, float *out) {
  if (n == 0 || !white || !out) return 1;
  Exposed e(n, alpha, std_, seed);
  e.fillBuffer();
  const std::complex<float> *w = e.white();
  const std::vector<float> &r = e.getFullBuffer();
  for (uint32_t m = 0; m < n; ++m) {
    white[m] = w[m].real();
    out[m] = r[m];
  }
  return 0;
}
}
