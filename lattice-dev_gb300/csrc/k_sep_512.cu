// k_sep_512.cu -- separable spectral passes for lines of 512 points.
#include "k_sep.cuh"

namespace lat {
int launch_sep_512(const SepArgs& a, int precision, int axis, cudaStream_t s) {
  return sep::sep_dispatch<512>(a, precision, axis, s);
}
int sep_columns_512(int precision, int nf) { return sep::sep_columns<512>(precision, nf); }
}  // namespace lat
