// k_sep_64.cu -- separable spectral passes for lines of 64 points.
#include "k_sep_stream.cuh"

namespace lat {
int launch_sep_64(const SepArgs& a, int precision, int axis, cudaStream_t s) {
  return sep::sep_dispatch<64>(a, precision, axis, s);
}
int sep_columns_64(int precision, int nf) { return sep::sep_columns<64>(precision, nf); }
// pairs of one-field runs (ensembles)
int launch_sep_runs_64(const SepArgs& a, int axis, cudaStream_t s) {
  return sep::sep_stream_dispatch<64, true>(a, axis, s);
}
int sep_runs_lines_64(int axis) { return sep::stream_lines<64>(axis); }
}  // namespace lat
