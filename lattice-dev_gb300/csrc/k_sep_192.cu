// k_sep_192.cu -- streamed separable passes for pairs of one-field runs on
// lines of 192 points (16 threads x 12-point register DFTs).
#include "k_sep_stream.cuh"

namespace lat {
int launch_sep_runs_192(const SepArgs& a, int axis, cudaStream_t s) {
  return sep::sep_stream_dispatch<192, true>(a, axis, s);
}
int sep_runs_lines_192(int axis) { return sep::stream_lines<192>(axis); }
}  // namespace lat
