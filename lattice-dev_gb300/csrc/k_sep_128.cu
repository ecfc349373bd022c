// k_sep_128.cu -- separable spectral passes for lines of 128 points.
#include "k_sep.cuh"

namespace lat {
int launch_sep_128(const SepArgs& a, int precision, int axis, cudaStream_t s) {
  return sep::sep_dispatch<128>(a, precision, axis, s);
}
int sep_columns_128(int precision, int nf) { return sep::sep_columns<128>(precision, nf); }
}  // namespace lat
