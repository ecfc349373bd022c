// k_sep_16.cu -- separable spectral passes for lines of 16 points.
#include "k_sep.cuh"

namespace lat {
int launch_sep_16(const SepArgs& a, int precision, int axis, cudaStream_t s) {
  return sep::sep_dispatch<16>(a, precision, axis, s);
}
int sep_columns_16(int precision, int nf) { return sep::sep_columns<16>(precision, nf); }
}  // namespace lat
