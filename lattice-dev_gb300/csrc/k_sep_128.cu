// k_sep_128.cu -- separable spectral passes for lines of 128 points.
#include "k_sep_stream.cuh"

namespace lat {
int launch_sep_128(const SepArgs& a, int precision, int axis, cudaStream_t s) {
  // two FP32 fields: the streamed passes when the lines form whole tiles
  if (precision == LAT_FP32_KAHAN && a.stream) {
    const int st = sep::sep_stream_dispatch<128>(a, axis, s);
    if (st != LAT_ERR_UNSUPPORTED) return st;
  }
  return sep::sep_dispatch<128>(a, precision, axis, s);
}
int sep_columns_128(int precision, int nf) { return sep::sep_columns<128>(precision, nf); }
}  // namespace lat
