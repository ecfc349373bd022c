// k_sep_32.cu -- separable spectral passes for lines of 32 points.
#include "k_sep.cuh"

namespace lat {
int launch_sep_32(const SepArgs& a, int precision, int axis, cudaStream_t s) {
  return sep::sep_dispatch<32>(a, precision, axis, s);
}
int sep_columns_32(int precision, int nf) { return sep::sep_columns<32>(precision, nf); }
}  // namespace lat
