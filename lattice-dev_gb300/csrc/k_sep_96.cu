// k_sep_96.cu -- streamed separable passes for pairs of one-field runs on
// lines of 96 points (8 threads x 12-point register DFTs).
#include "k_sep_stream.cuh"

namespace lat {
int launch_sep_runs_96(const SepArgs& a, int axis, cudaStream_t s) {
  return sep::sep_stream_dispatch<96, true>(a, axis, s);
}
int sep_runs_lines_96(int axis) { return sep::stream_lines<96>(axis); }
}  // namespace lat
