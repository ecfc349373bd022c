// k_sep_128.cu -- separable spectral passes for lines of 128 points.
#include "k_sep_stream.cuh"

namespace lat {
int launch_sep_128(const SepArgs& a, int precision, int axis, cudaStream_t s) {
  // two FP32 fields on a lattice whose passes all form whole tiles (the
  // streamed passes keep zs, not the Laplacian, between passes)
  if (a.stream) return sep::sep_stream_dispatch<128, false>(a, axis, s);
  return sep::sep_dispatch<128>(a, precision, axis, s);
}
int sep_stream_lines_128(int axis) { return sep::stream_lines<128>(axis); }
int sep_columns_128(int precision, int nf) { return sep::sep_columns<128>(precision, nf); }
// pairs of one-field runs (ensembles)
int launch_sep_runs_128(const SepArgs& a, int axis, cudaStream_t s) {
  return sep::sep_stream_dispatch<128, true>(a, axis, s);
}
int sep_runs_lines_128(int axis) { return sep::stream_lines<128>(axis); }
}  // namespace lat
