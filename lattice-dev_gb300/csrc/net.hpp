// net.hpp -- launchers of the closure network kernels (k_net.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "engine.hpp"

namespace lat {
namespace net {

enum Epi { EPI_GELU = 0, EPI_LINEAR = 1, EPI_BWD = 2 };

// Layer geometry: inputs padded 4 -> 8 channels, outputs 2 -> 8.
constexpr int C_IN = 8, C_HID = 32, C_OUT = 8;
constexpr int64_t W1_N = 27LL * C_IN * C_HID, W2_N = 27LL * C_HID * C_HID, W3_N = 27LL * C_HID * C_OUT;
// flat parameter vector: W1 b1 W2 b2 W3 b3
constexpr int64_t OFF_W1 = 0, OFF_B1 = OFF_W1 + W1_N, OFF_W2 = OFF_B1 + C_HID, OFF_B2 = OFF_W2 + W2_N,
                  OFF_W3 = OFF_B2 + C_HID, OFF_B3 = OFF_W3 + W3_N, N_PARAMS = OFF_B3 + C_OUT;

struct ConvArgs {
  int nx, ny, nz;
  int64_t nlat;                 // lattices in the batch
  const __nv_bfloat16* in;      // [nlat][N][CA]
  const __nv_bfloat16* w;       // [27][CB][CA]
  const float* bias;            // [CB] (forward) or null
  __nv_bfloat16* out;           // [nlat][N][CB] (GELU, BWD)
  __nv_bfloat16* zout;          // pre-activation (GELU, optional)
  const __nv_bfloat16* zin;     // pre-activation of the layer (BWD)
  float* outf;                  // [nlat][N][2] (LINEAR)
  int* err;                     // device error word (bounded waits of the tensor-memory kernel)
};

struct WgradArgs {
  int nx, ny, nz;
  int64_t nlat;
  const __nv_bfloat16* x;  // [nlat][N][CX] layer input (shifted by the taps)
  const __nv_bfloat16* d;  // [nlat][N][CD] gradient at the layer's pre-activation
  float* part;             // [nblk][27][CX][CD]
  float* part_b;           // [nblk][CD]
};

struct PackArgs {
  const void* ch[4];   // channel arrays (FP32 or FP64), lattice l at ch[c] + idx[l] * lat_stride
  const int32_t* idx;  // [nlat] or null (lattice l at offset l * lat_stride)
  int64_t lat_stride, nlat, N;
  double shift[4], scale[4];
  const DevScalars* sc;  // conformal units: fields times a, momenta over a (a from the scalar block)
  double hg;             // a gravity half-step still to apply: a - hg ysclp / 6
  __nv_bfloat16* out;    // [nlat][N][8]
};

struct LossArgs {
  const float* out;      // [nlat][N][2]
  const float* t0;       // target channel 0 of sample 0 (sample idx[l] at + idx[l] * lat_stride)
  const float* t1;
  double tscale[2];
  const int32_t* idx;
  int64_t lat_stride, nlat, N;
  __nv_bfloat16* dout;   // [nlat][N][8]
  double* part;          // [nblk]
};

struct CorrArgs {
  void* pi;            // [2][N] momenta (FP32 or FP64)
  const float* out;    // [N][2] network output
  double tscale[2];
  double hk;
  int conf;
  int units;  // 0: Delta in program variables (factor a^4); 1: a^3 Delta (factor a)
  const DevScalars* sc;
  int64_t N;
};

// activations of one forward pass (z1, z2 only when training)
struct InferBufs {
  __nv_bfloat16 *a0, *z1, *a1, *z2, *a2;
  float* out;  // [nlat][N][2]
};

// forward pass of one lattice from four channel arrays (phi, chi, pi_phi, pi_chi)
// (conformal units: hg is a gravity half-step the scale factor has still to take)
int infer(lat_net_s* n, const void* const ch[4], int fp64, int nx, int ny, int nz, const DevScalars* conformal_sc,
          double hg, const InferBufs& b, cudaStream_t s);
void out_scale(const lat_net_s* n, double out[2]);
int net_device(const lat_net_s* n);
int* net_err(const lat_net_s* n);
void net_attach_ref(lat_net_s* n, int delta);
uint64_t net_key(const lat_net_s* n);  // changes with every network and every normalisation

int conv(const ConvArgs& a, int ca, int cb, int epi, int nsm, cudaStream_t s);
// layers with 32 output channels on tcgen05 (k_conv_tc.cu): 32 -> 32 (forward and
// backward data) and the 8-channel (4 padded) input layer; nx % 64 == 0 (rows of 128 or 64 sites)
bool conv_tc_ok(int ca, int cb, int epi, int nx, int ny);
int conv_tc(const ConvArgs& a, int ca, int epi, int nsm, int* err, cudaStream_t s);
int wgrad_blocks(int nsm);
int wgrad(const WgradArgs& a, int cx, int cd, int nblk, float* dW, float* db, cudaStream_t s);
int pack(const PackArgs& a, int fp64, int nsm, cudaStream_t s);
int loss(const LossArgs& a, int nblk, double* out, cudaStream_t s);
int adam(float* p, const float* g, float* m, float* v, int64_t n, double lr, int64_t step, cudaStream_t s);
int repack(const float* W, int ci, int co, __nv_bfloat16* fwd, __nv_bfloat16* bwd, cudaStream_t s);
int corr_kick(const CorrArgs& a, int fp64, int nsm, cudaStream_t s);

}  // namespace net
}  // namespace lat
