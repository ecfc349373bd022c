// k_sep_256.cu -- separable spectral passes for lines of 256 points.
#include "k_sep.cuh"

namespace lat {
int launch_sep_256(const SepArgs& a, int precision, int axis, cudaStream_t s) {
  return sep::sep_dispatch<256>(a, precision, axis, s);
}
int sep_columns_256(int precision, int nf) { return sep::sep_columns<256>(precision, nf); }
}  // namespace lat
