// net.cu -- host side of the learned subgrid closure: parameters, training
// step, inference, and the C ABI of include/lattice.h (lat_net_*).
//
// The closure has no counterpart in the reference (it is an addition on top
// of the reference's coarse-lattice evolution).  A network maps the coarse
// fields and momenta (phi, chi, pi_phi, pi_chi) at a kick to a correction of
// the two forces: the kick uses V'(phi) - Delta, with Delta trained on
// V'(F phi) - F V'(phi) of sharp-k filtered fine-lattice runs (lat_coarsen).
#include <atomic>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "net.hpp"

using namespace lat;
using namespace lat::net;

#define NCK(x)                                       \
  do {                                               \
    cudaError_t e_ = (x);                            \
    if (e_ != cudaSuccess) return cuda_fail(e_, #x); \
  } while (0)
#define NRET(x)                  \
  do {                           \
    int s_ = (x);                \
    if (s_ != LAT_OK) return s_; \
  } while (0)

struct lat_net_s {
  int dev = 0, nsm = 152;
  cudaStream_t stream = nullptr;
  float *P = nullptr, *G = nullptr, *m = nullptr, *v = nullptr;  // flat FP32 parameters, gradient, Adam moments
  int64_t step = 0;
  __nv_bfloat16 *wf1 = nullptr, *wf2 = nullptr, *wf3 = nullptr, *wb2 = nullptr, *wb3 = nullptr;
  double shift[4] = {0, 0, 0, 0}, scale[4] = {1, 1, 1, 1}, tscale[2] = {1, 1};
  // training activations, sized for `cap` sites
  int64_t cap = 0;
  __nv_bfloat16 *a0 = nullptr, *z1 = nullptr, *a1 = nullptr, *z2 = nullptr, *a2 = nullptr;
  __nv_bfloat16 *d3 = nullptr, *d2 = nullptr, *d1 = nullptr;
  float* out = nullptr;
  float *part = nullptr, *part_b = nullptr;
  double *lpart = nullptr, *lsum = nullptr;
  int32_t* idx = nullptr;
  int idx_cap = 0;
  int64_t launches = 0;
  int* err = nullptr;  // device error word of the tensor-memory convolutions (bounded waits)
  int attached = 0;    // lattices this network is attached to (lat_closure_attach)
  uint64_t key = 0;    // unique per network and normalisation (kernel arguments captured in graphs)
};

namespace {

std::atomic<uint64_t> g_net_keys{0};

struct Guard {
  explicit Guard(lat_net_s* n) {
    cudaSetDevice(n->dev);
    g_launch_counter = &n->launches;
  }
  ~Guard() { g_launch_counter = nullptr; }
};

void free_acts(lat_net_s* n) {
  void* ps[] = {n->a0, n->z1, n->a1, n->z2, n->a2, n->d3, n->d2, n->d1, n->out};
  for (void* p : ps)
    if (p) cudaFree(p);
  n->a0 = n->z1 = n->a1 = n->z2 = n->a2 = n->d3 = n->d2 = n->d1 = nullptr;
  n->out = nullptr;
  n->cap = 0;
}

int ensure_acts(lat_net_s* n, int64_t sites) {
  if (sites <= n->cap) return LAT_OK;
  NCK(cudaStreamSynchronize(n->stream));
  free_acts(n);
  const size_t b8 = (size_t)sites * C_IN * 2, b32 = (size_t)sites * C_HID * 2;
  NCK(cudaMalloc(&n->a0, b8));
  NCK(cudaMalloc(&n->z1, b32));
  NCK(cudaMalloc(&n->a1, b32));
  NCK(cudaMalloc(&n->z2, b32));
  NCK(cudaMalloc(&n->a2, b32));
  NCK(cudaMalloc(&n->d3, b8));
  NCK(cudaMalloc(&n->d2, b32));
  NCK(cudaMalloc(&n->d1, b32));
  NCK(cudaMalloc(&n->out, (size_t)sites * 2 * sizeof(float)));
  n->cap = sites;
  return LAT_OK;
}

int ensure_idx(lat_net_s* n, const int32_t* idx_host, int nidx) {
  if (nidx > n->idx_cap) {
    NCK(cudaStreamSynchronize(n->stream));
    if (n->idx) cudaFree(n->idx);
    NCK(cudaMalloc(&n->idx, (size_t)nidx * sizeof(int32_t)));
    n->idx_cap = nidx;
  }
  NCK(cudaMemcpyAsync(n->idx, idx_host, (size_t)nidx * sizeof(int32_t), cudaMemcpyHostToDevice, n->stream));
  return LAT_OK;
}

int repack_all(lat_net_s* n, cudaStream_t s) {
  NRET(repack(n->P + OFF_W1, C_IN, C_HID, n->wf1, nullptr, s));
  NRET(repack(n->P + OFF_W2, C_HID, C_HID, n->wf2, n->wb2, s));
  NRET(repack(n->P + OFF_W3, C_HID, C_OUT, n->wf3, n->wb3, s));
  return LAT_OK;
}

// splitmix64 stream for the initial weights
uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

int check_lattice(int nx, int ny, int nz) {
  if (nx < 16 || ny < 8 || nz < 1 || nx % 16 || ny % 8)
    return set_error(LAT_ERR_ARG, "closure lattice: nx a multiple of 16, ny a multiple of 8");
  return LAT_OK;
}

// forward pass over nlat lattices whose input is already in n->a0 (or b.a0)
int forward(lat_net_s* n, const InferBufs& b, int nx, int ny, int nz, int64_t nlat, bool store_z, cudaStream_t s) {
  ConvArgs c{};
  c.nx = nx; c.ny = ny; c.nz = nz; c.nlat = nlat;
  c.err = n->err;
  c.in = b.a0; c.w = n->wf1; c.bias = n->P + OFF_B1; c.out = b.a1; c.zout = store_z ? b.z1 : nullptr;
  NRET(conv(c, C_IN, C_HID, EPI_GELU, n->nsm, s));
  c.in = b.a1; c.w = n->wf2; c.bias = n->P + OFF_B2; c.out = b.a2; c.zout = store_z ? b.z2 : nullptr;
  NRET(conv(c, C_HID, C_HID, EPI_GELU, n->nsm, s));
  c.in = b.a2; c.w = n->wf3; c.bias = n->P + OFF_B3; c.out = nullptr; c.zout = nullptr; c.outf = b.out;
  NRET(conv(c, C_HID, C_OUT, EPI_LINEAR, n->nsm, s));
  return LAT_OK;
}

InferBufs train_bufs(lat_net_s* n) {
  InferBufs b{};
  b.a0 = n->a0; b.z1 = n->z1; b.a1 = n->a1; b.z2 = n->z2; b.a2 = n->a2; b.out = n->out;
  return b;
}

int pack_samples(lat_net_s* n, const float* data, int64_t stride, int64_t N, int nidx, cudaStream_t s) {
  PackArgs p{};
  for (int c = 0; c < 4; ++c) {
    p.ch[c] = data + (int64_t)c * N;
    p.shift[c] = n->shift[c];
    p.scale[c] = n->scale[c];
  }
  p.idx = n->idx;
  p.lat_stride = stride;
  p.nlat = nidx;
  p.N = N;
  p.out = n->a0;
  return pack(p, 0, n->nsm, s);
}

// loss and gradients of the batch; leaves the gradient in n->G
int loss_and_grad(lat_net_s* n, const float* data, int64_t stride, int nidx, int nx, int ny, int nz, double* loss) {
  const int64_t N = (int64_t)nx * ny * nz;
  cudaStream_t s = n->stream;
  NRET(pack_samples(n, data, stride, N, nidx, s));
  InferBufs b = train_bufs(n);
  NRET(forward(n, b, nx, ny, nz, nidx, true, s));
  LossArgs la{};
  la.out = n->out;
  la.t0 = data + 4 * N;
  la.t1 = data + 5 * N;
  la.tscale[0] = n->tscale[0];
  la.tscale[1] = n->tscale[1];
  la.idx = n->idx;
  la.lat_stride = stride;
  la.nlat = nidx;
  la.N = N;
  la.dout = n->d3;
  la.part = n->lpart;
  NRET(lat::net::loss(la, 2 * n->nsm, n->lsum, s));
  const int nblk = wgrad_blocks(n->nsm);
  WgradArgs w{};
  w.nx = nx; w.ny = ny; w.nz = nz; w.nlat = nidx;
  w.part = n->part;
  w.part_b = n->part_b;
  // layer 3: input a2, gradient d3
  w.x = n->a2; w.d = n->d3;
  NRET(wgrad(w, C_HID, C_OUT, nblk, n->G + OFF_W3, n->G + OFF_B3, s));
  ConvArgs c{};
  c.nx = nx; c.ny = ny; c.nz = nz; c.nlat = nidx;
  c.err = n->err;
  c.in = n->d3; c.w = n->wb3; c.zin = n->z2; c.out = n->d2;
  NRET(conv(c, C_OUT, C_HID, EPI_BWD, n->nsm, s));
  // layer 2
  w.x = n->a1; w.d = n->d2;
  NRET(wgrad(w, C_HID, C_HID, nblk, n->G + OFF_W2, n->G + OFF_B2, s));
  c.in = n->d2; c.w = n->wb2; c.zin = n->z1; c.out = n->d1;
  NRET(conv(c, C_HID, C_HID, EPI_BWD, n->nsm, s));
  // layer 1
  w.x = n->a0; w.d = n->d1;
  NRET(wgrad(w, C_IN, C_HID, nblk, n->G + OFF_W1, n->G + OFF_B1, s));
  if (loss) {
    NCK(cudaMemcpyAsync(loss, n->lsum, sizeof(double), cudaMemcpyDeviceToHost, s));
  }
  NCK(cudaStreamSynchronize(s));
  return LAT_OK;
}

// the error word of the bounded waits, read after the stream has drained
int check_err(lat_net_s* n) {
  int h = 0;
  NCK(cudaMemcpyAsync(&h, n->err, sizeof(int), cudaMemcpyDeviceToHost, n->stream));
  NCK(cudaStreamSynchronize(n->stream));
  if (h) {
    cudaMemsetAsync(n->err, 0, sizeof(int), n->stream);
    cudaStreamSynchronize(n->stream);
    return set_error(LAT_ERR_TIMEOUT, "closure convolution: a tensor-core wait gave up");
  }
  return LAT_OK;
}

int batch_args(lat_net_s* n, const float* data, int64_t stride, const int32_t* idx, int32_t nidx, int nx, int ny,
               int nz) {
  if (!n || !data || !idx || nidx < 1) return set_error(LAT_ERR_ARG, "null argument or empty batch");
  NRET(check_lattice(nx, ny, nz));
  const int64_t N = (int64_t)nx * ny * nz;
  if (stride < 6 * N) return set_error(LAT_ERR_ARG, "sample stride below 6 channels x sites");
  NRET(ensure_acts(n, N * nidx));
  NRET(ensure_idx(n, idx, nidx));
  return LAT_OK;
}

}  // namespace

namespace lat {
namespace net {

int infer(lat_net_s* n, const void* const ch[4], int fp64, int nx, int ny, int nz, const DevScalars* conformal_sc,
          double hg, const InferBufs& b, cudaStream_t s) {
  PackArgs p{};
  p.sc = conformal_sc;
  p.hg = hg;
  for (int c = 0; c < 4; ++c) {
    p.ch[c] = ch[c];
    p.shift[c] = n->shift[c];
    p.scale[c] = n->scale[c];
  }
  p.idx = nullptr;
  p.lat_stride = 0;
  p.nlat = 1;
  p.N = (int64_t)nx * ny * nz;
  p.out = b.a0;
  NRET(pack(p, fp64, n->nsm, s));
  return forward(n, b, nx, ny, nz, 1, false, s);
}

void out_scale(const lat_net_s* n, double out[2]) {
  out[0] = n->tscale[0];
  out[1] = n->tscale[1];
}

int net_device(const lat_net_s* n) { return n->dev; }

int* net_err(const lat_net_s* n) { return n->err; }

void net_attach_ref(lat_net_s* n, int delta) { n->attached += delta; }

uint64_t net_key(const lat_net_s* n) { return n->key; }

}  // namespace net
}  // namespace lat

extern "C" {

int64_t lat_net_nparams(void) { return N_PARAMS; }

int lat_net_create(lat_net_t** out, int32_t device, uint64_t seed) {
  if (!out) return set_error(LAT_ERR_ARG, "null output");
  *out = nullptr;
  lat_net_s* n = new lat_net_s();
  n->dev = device;
  n->key = ++g_net_keys;
  Guard g(n);
  auto bail = [&](int st) {
    lat_net_destroy(n);
    return st;
  };
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return bail(cuda_fail(e, "cudaSetDevice"));
  cudaDeviceGetAttribute(&n->nsm, cudaDevAttrMultiProcessorCount, device);
  if ((e = cudaStreamCreateWithFlags(&n->stream, cudaStreamNonBlocking)) != cudaSuccess)
    return bail(cuda_fail(e, "stream"));
  const size_t pb = (size_t)N_PARAMS * sizeof(float);
  float** fl[] = {&n->P, &n->G, &n->m, &n->v};
  for (float** p : fl) {
    if ((e = cudaMalloc(p, pb)) != cudaSuccess) return bail(cuda_fail(e, "parameters"));
    cudaMemsetAsync(*p, 0, pb, n->stream);
  }
  __nv_bfloat16** bl[] = {&n->wf1, &n->wf2, &n->wf3, &n->wb2, &n->wb3};
  const int64_t bn[] = {W1_N, W2_N, W3_N, W2_N, W3_N};
  for (int i = 0; i < 5; ++i)
    if ((e = cudaMalloc(bl[i], (size_t)bn[i] * 2)) != cudaSuccess) return bail(cuda_fail(e, "bf16 weights"));
  const int nblk = wgrad_blocks(n->nsm);
  if ((e = cudaMalloc(&n->part, (size_t)nblk * 27 * C_HID * C_HID * sizeof(float))) != cudaSuccess ||
      (e = cudaMalloc(&n->part_b, (size_t)nblk * C_HID * sizeof(float))) != cudaSuccess ||
      (e = cudaMalloc(&n->lpart, (size_t)2 * n->nsm * sizeof(double))) != cudaSuccess ||
      (e = cudaMalloc(&n->lsum, sizeof(double))) != cudaSuccess ||
      (e = cudaMalloc(&n->err, sizeof(int))) != cudaSuccess)
    return bail(cuda_fail(e, "training scratch"));
  cudaMemsetAsync(n->err, 0, sizeof(int), n->stream);
  // He-normal initial weights (Box-Muller on a splitmix64 stream); the last
  // layer starts 100x smaller so the untrained closure is close to zero.
  // Padded channels (inputs 4..7, outputs 2..7) stay zero.
  std::vector<float> h(N_PARAMS, 0.f);
  uint64_t ctr = 0;
  auto gauss = [&]() {
    const double u1 = ((mix64(seed * 0x100000001B3ULL + ctr++) >> 11) + 1) * 0x1.0p-53;
    const double u2 = ((mix64(seed * 0x100000001B3ULL + ctr++) >> 11) + 1) * 0x1.0p-53;
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
  };
  for (int tap = 0; tap < 27; ++tap)
    for (int i = 0; i < C_IN; ++i)
      for (int o = 0; o < C_HID; ++o)
        h[OFF_W1 + (tap * C_IN + i) * C_HID + o] = i < 4 ? (float)(gauss() * std::sqrt(2.0 / (27 * 4))) : 0.f;
  for (int64_t k = 0; k < W2_N; ++k) h[OFF_W2 + k] = (float)(gauss() * std::sqrt(2.0 / (27 * C_HID)));
  for (int tap = 0; tap < 27; ++tap)
    for (int i = 0; i < C_HID; ++i)
      for (int o = 0; o < C_OUT; ++o)
        h[OFF_W3 + (tap * C_HID + i) * C_OUT + o] = o < 2 ? (float)(0.01 * gauss() * std::sqrt(1.0 / (27 * C_HID))) : 0.f;
  if ((e = cudaMemcpyAsync(n->P, h.data(), pb, cudaMemcpyHostToDevice, n->stream)) != cudaSuccess)
    return bail(cuda_fail(e, "initial weights"));
  int st = repack_all(n, n->stream);
  if (st != LAT_OK) return bail(st);
  if ((e = cudaStreamSynchronize(n->stream)) != cudaSuccess) return bail(cuda_fail(e, "create sync"));
  *out = n;
  return LAT_OK;
}

int lat_net_destroy(lat_net_t* n) {
  if (!n) return LAT_OK;
  if (n->attached > 0) return set_error(LAT_ERR_STATE, "network still attached to a lattice: detach it first");
  cudaSetDevice(n->dev);
  if (n->stream) cudaStreamSynchronize(n->stream);
  free_acts(n);
  void* ps[] = {n->P, n->G, n->m, n->v, n->wf1, n->wf2, n->wf3, n->wb2, n->wb3,
                n->part, n->part_b, n->lpart, n->lsum, n->idx, n->err};
  for (void* p : ps)
    if (p) cudaFree(p);
  if (n->stream) cudaStreamDestroy(n->stream);
  delete n;
  return LAT_OK;
}

int lat_net_get_params(lat_net_t* n, float* out, int64_t count) {
  if (!n || !out) return set_error(LAT_ERR_ARG, "null argument");
  if (count != N_PARAMS) return set_error(LAT_ERR_ARG, "parameter count mismatch");
  Guard g(n);
  NCK(cudaMemcpyAsync(out, n->P, (size_t)N_PARAMS * sizeof(float), cudaMemcpyDeviceToHost, n->stream));
  NCK(cudaStreamSynchronize(n->stream));
  return LAT_OK;
}

int lat_net_set_params(lat_net_t* n, const float* in, int64_t count) {
  if (!n || !in) return set_error(LAT_ERR_ARG, "null argument");
  if (count != N_PARAMS) return set_error(LAT_ERR_ARG, "parameter count mismatch");
  Guard g(n);
  NCK(cudaMemcpyAsync(n->P, in, (size_t)N_PARAMS * sizeof(float), cudaMemcpyHostToDevice, n->stream));
  NRET(repack_all(n, n->stream));
  NCK(cudaStreamSynchronize(n->stream));
  return LAT_OK;
}

int lat_net_set_norm(lat_net_t* n, const double in_shift[4], const double in_scale[4], const double out_scale[2]) {
  if (!n || !in_shift || !in_scale || !out_scale) return set_error(LAT_ERR_ARG, "null argument");
  for (int c = 0; c < 4; ++c) {
    n->shift[c] = in_shift[c];
    n->scale[c] = in_scale[c];
  }
  if (out_scale[0] == 0.0 || out_scale[1] == 0.0) return set_error(LAT_ERR_ARG, "zero output scale");
  n->tscale[0] = out_scale[0];
  n->tscale[1] = out_scale[1];
  n->key = ++g_net_keys;  // graphs captured with the old normalisation no longer match
  return LAT_OK;
}

int lat_net_get_norm(const lat_net_t* n, double in_shift[4], double in_scale[4], double out_scale[2]) {
  if (!n || !in_shift || !in_scale || !out_scale) return set_error(LAT_ERR_ARG, "null argument");
  for (int c = 0; c < 4; ++c) {
    in_shift[c] = n->shift[c];
    in_scale[c] = n->scale[c];
  }
  out_scale[0] = n->tscale[0];
  out_scale[1] = n->tscale[1];
  return LAT_OK;
}

int lat_net_forward(lat_net_t* n, const float* data, int64_t stride, const int32_t* idx, int32_t nidx, int32_t nx,
                    int32_t ny, int32_t nz, float* out_dev) {
  if (!out_dev) return set_error(LAT_ERR_ARG, "null output");
  if (!n) return set_error(LAT_ERR_ARG, "null network");
  Guard g(n);
  NRET(batch_args(n, data, stride, idx, nidx, nx, ny, nz));
  const int64_t N = (int64_t)nx * ny * nz;
  NRET(pack_samples(n, data, stride, N, nidx, n->stream));
  InferBufs b = train_bufs(n);
  b.out = out_dev;
  NRET(forward(n, b, nx, ny, nz, nidx, false, n->stream));
  return check_err(n);
}

int lat_net_grad(lat_net_t* n, const float* data, int64_t stride, const int32_t* idx, int32_t nidx, int32_t nx,
                 int32_t ny, int32_t nz, double* loss, float* grad_host) {
  if (!n) return set_error(LAT_ERR_ARG, "null network");
  Guard g(n);
  NRET(batch_args(n, data, stride, idx, nidx, nx, ny, nz));
  NRET(loss_and_grad(n, data, stride, nidx, nx, ny, nz, loss));
  NRET(check_err(n));
  if (grad_host) {
    NCK(cudaMemcpyAsync(grad_host, n->G, (size_t)N_PARAMS * sizeof(float), cudaMemcpyDeviceToHost, n->stream));
    NCK(cudaStreamSynchronize(n->stream));
  }
  return LAT_OK;
}

int lat_net_train_step(lat_net_t* n, const float* data, int64_t stride, const int32_t* idx, int32_t nidx,
                       int32_t nx, int32_t ny, int32_t nz, double lr, double* loss) {
  if (!n) return set_error(LAT_ERR_ARG, "null network");
  if (!(lr > 0.0)) return set_error(LAT_ERR_ARG, "learning rate must be positive");
  Guard g(n);
  NRET(batch_args(n, data, stride, idx, nidx, nx, ny, nz));
  NRET(loss_and_grad(n, data, stride, nidx, nx, ny, nz, loss));
  n->step += 1;
  NRET(adam(n->P, n->G, n->m, n->v, N_PARAMS, lr, n->step, n->stream));
  NRET(repack_all(n, n->stream));
  return check_err(n);
}

int64_t lat_net_launch_count(const lat_net_t* n) { return n ? n->launches : -1; }

int lat_net_time_forward(lat_net_t* n, int32_t nx, int32_t ny, int32_t nz, int32_t reps, double ms[4]) {
  if (!n || !ms || reps < 1) return set_error(LAT_ERR_ARG, "bad argument");
  Guard g(n);
  NRET(check_lattice(nx, ny, nz));
  const int64_t N = (int64_t)nx * ny * nz;
  NRET(ensure_acts(n, N));
  NCK(cudaMemsetAsync(n->a0, 0, (size_t)N * C_IN * 2, n->stream));
  cudaEvent_t ev[5];
  for (auto& e : ev) NCK(cudaEventCreate(&e));
  InferBufs b = train_bufs(n);
  ConvArgs c{};
  c.nx = nx; c.ny = ny; c.nz = nz; c.nlat = 1;
  c.err = n->err;
  double acc[4] = {0, 0, 0, 0};
  int st = LAT_OK;
  for (int r = 0; r <= reps && st == LAT_OK; ++r) {  // r = 0 is a warm-up
    PackArgs p{};
    for (int q = 0; q < 4; ++q) {
      p.ch[q] = n->d2;  // any device array of N floats: the timing does not look at values
      p.scale[q] = 1.0;
    }
    p.nlat = 1;
    p.N = N;
    p.out = b.a0;
    cudaEventRecord(ev[0], n->stream);
    if ((st = pack(p, 0, n->nsm, n->stream)) != LAT_OK) break;
    cudaEventRecord(ev[1], n->stream);
    c.in = b.a0; c.w = n->wf1; c.bias = n->P + OFF_B1; c.out = b.a1; c.zout = nullptr;
    if ((st = conv(c, C_IN, C_HID, EPI_GELU, n->nsm, n->stream)) != LAT_OK) break;
    cudaEventRecord(ev[2], n->stream);
    c.in = b.a1; c.w = n->wf2; c.bias = n->P + OFF_B2; c.out = b.a2;
    if ((st = conv(c, C_HID, C_HID, EPI_GELU, n->nsm, n->stream)) != LAT_OK) break;
    cudaEventRecord(ev[3], n->stream);
    c.in = b.a2; c.w = n->wf3; c.bias = n->P + OFF_B3; c.out = nullptr; c.outf = b.out;
    if ((st = conv(c, C_HID, C_OUT, EPI_LINEAR, n->nsm, n->stream)) != LAT_OK) break;
    cudaEventRecord(ev[4], n->stream);
    cudaEventSynchronize(ev[4]);
    if (r == 0) continue;
    for (int q = 0; q < 4; ++q) {
      float t = 0;
      cudaEventElapsedTime(&t, ev[q], ev[q + 1]);
      acc[q] += t;
    }
  }
  for (auto& e : ev) cudaEventDestroy(e);
  if (st != LAT_OK) return st;
  NRET(check_err(n));
  for (int q = 0; q < 4; ++q) ms[q] = acc[q] / reps;
  return LAT_OK;
}

}  // extern "C"
