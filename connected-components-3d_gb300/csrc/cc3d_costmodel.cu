// cc3d_costmodel.cu -- volume features and the learned cost model.
//
// The cost model predicts, from 16 cheap features of a volume, the log of the
// labelling time of every tile-pass configuration (CC3D_TILE_CONFIGS outputs),
// so that a configuration can be chosen without timing them all.  It is a
// small FP32 MLP, 16 -> 64 -> 64 -> 12 with ReLU, trained on timings the
// autotuner itself produces.  Training (mini-batch Adam on a squared error
// over the measured outputs) and inference are the kernels below; the
// features are sampled on the device.  It never affects labels: every
// configuration labels identically.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "cc3d_gpu.h"
#include "cc3d_internal.h"

using namespace cc3dgpu;

namespace {

constexpr int NF = CC3D_COST_FEATURES;  // 16
constexpr int NH = 64;
constexpr int NO = CC3D_TILE_CONFIGS;  // 12: variant x tile shape x load path
// parameter layout: W1[NF][NH] b1[NH] W2[NH][NH] b2[NH] W3[NH][NO] b3[NO]
constexpr int OW1 = 0, OB1 = OW1 + NF * NH, OW2 = OB1 + NH, OB2 = OW2 + NH * NH, OW3 = OB2 + NH,
              OB3 = OW3 + NH * NO, NPARAM = OB3 + NO;
// normalisation after the weights: feature mean/std, output mean/std
constexpr int OFM = NPARAM, OFS = OFM + NF, OOM = OFS + NF, OOS = OOM + NO, NTOTAL = OOS + NO;
static_assert(NTOTAL == CC3D_COST_PARAMS, "parameter count");

int failf(int code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
int failf(int code, const char* fmt, ...) {
  char buf[256];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  return api_fail(code, buf);
}

#define CKC(call)                                                                                \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess) return failf(CC3D_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

// ------------------------------------------------------------ features
constexpr int kSamples = 1 << 16;   // sampled voxels
constexpr int kDistinct = 4096;     // of which the first ones are kept for the distinct count

struct FeatureSums {
  unsigned long long fg, same_x, same_y, same_z, start_x, valid_x, valid_y, valid_z;
};

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
  // splitmix64 finaliser: a well-spread sample index from a counter
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

template <typename T>
__global__ void __launch_bounds__(256) k_features(const T* in, int64_t sx, int64_t sy, int64_t sz,
                                                  FeatureSums* sums, unsigned long long* distinct) {
  const int64_t voxels = sx * sy * sz;
  unsigned long long fg = 0, sxn = 0, syn = 0, szn = 0, st = 0, vx = 0, vy = 0, vz = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kSamples; i += gridDim.x * blockDim.x) {
    const int64_t idx = (int64_t)(mix64((uint64_t)i) % (uint64_t)voxels);
    const int64_t x = idx % sx, y = (idx / sx) % sy, z = idx / (sx * sy);
    const T v = in[idx];
    if (i < kDistinct) {
      unsigned long long bits = 0;
      memcpy(&bits, &v, sizeof(T));
      distinct[i] = bits;
    }
    if (v == T(0)) continue;
    ++fg;
    if (x + 1 < sx) { ++vx; sxn += in[idx + 1] == v; }
    if (x > 0) st += in[idx - 1] != v;
    else ++st;
    if (y + 1 < sy) { ++vy; syn += in[idx + sx] == v; }
    if (z + 1 < sz) { ++vz; szn += in[idx + sx * sy] == v; }
  }
  unsigned long long a[8] = {fg, sxn, syn, szn, st, vx, vy, vz};
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    for (int o = 16; o > 0; o >>= 1) a[k] += __shfl_down_sync(FULL, a[k], o);
  }
  if ((threadIdx.x & 31) == 0) {
    unsigned long long* out = reinterpret_cast<unsigned long long*>(sums);
#pragma unroll
    for (int k = 0; k < 8; ++k)
      if (a[k]) atomicAdd(out + k, a[k]);
  }
}

// distinct values among the first kDistinct samples: one block sorts them
// (bitonic, shared memory) and counts the value changes
__global__ void __launch_bounds__(1024) k_distinct(unsigned long long* vals, int n, unsigned int* count) {
  __shared__ unsigned long long s[kDistinct];
  for (int i = threadIdx.x; i < kDistinct; i += blockDim.x) s[i] = i < n ? vals[i] : ~0ull;
  __syncthreads();
  for (int k = 2; k <= kDistinct; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < kDistinct; i += blockDim.x) {
        const int l = i ^ j;
        if (l > i) {
          const bool up = (i & k) == 0;
          const unsigned long long a = s[i], b = s[l];
          if ((a > b) == up) { s[i] = b; s[l] = a; }
        }
      }
      __syncthreads();
    }
  }
  unsigned int c = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) c += (i == 0 || s[i] != s[i - 1]) ? 1u : 0u;
  atomicAdd(count, c);
}

// ------------------------------------------------------------ the MLP
// forward of one dense layer for a mini-batch: Y[b][o] = act(sum_i X[b][i] W[i][o] + bias[o])
__global__ void k_dense_fwd(const float* X, const float* W, const float* bias, float* Y, int B, int I, int O,
                            int relu) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= B * O) return;
  const int b = t / O, o = t % O;
  float acc = bias[o];
  for (int i = 0; i < I; ++i) acc = fmaf(X[b * I + i], W[i * O + o], acc);
  Y[t] = relu ? fmaxf(acc, 0.f) : acc;
}

// dX[b][i] = sum_o dY[b][o] W[i][o], masked by the ReLU of the layer that made X
__global__ void k_dense_bwd_x(const float* dY, const float* W, const float* X, float* dX, int B, int I, int O) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= B * I) return;
  const int b = t / I, i = t % I;
  float acc = 0.f;
  for (int o = 0; o < O; ++o) acc = fmaf(dY[b * O + o], W[i * O + o], acc);
  dX[t] = X[t] > 0.f ? acc : 0.f;
}

// dW[i][o] = sum_b X[b][i] dY[b][o] / B; db[o] = sum_b dY[b][o] / B
__global__ void k_dense_bwd_w(const float* X, const float* dY, float* dW, float* db, int B, int I, int O) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < I * O) {
    const int i = t / O, o = t % O;
    float acc = 0.f;
    for (int b = 0; b < B; ++b) acc = fmaf(X[b * I + i], dY[b * O + o], acc);
    dW[t] = acc / B;
  } else if (t < I * O + O) {
    const int o = t - I * O;
    float acc = 0.f;
    for (int b = 0; b < B; ++b) acc += dY[b * O + o];
    db[o] = acc / B;
  }
}

// squared error over the measured outputs (mask 1) and its gradient 2 (p - y); the
// weight gradients average over the mini-batch
__global__ void k_loss(const float* P, const float* Y, const float* M, float* dP, float* loss, int n) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const float d = (P[t] - Y[t]) * M[t];
  dP[t] = 2.f * d;
  atomicAdd(loss, d * d);
}

__global__ void k_adam(float* p, const float* g, float* m, float* v, int n, float lr, float b1, float b2,
                       float c1, float c2) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const float gt = g[t];
  const float mt = b1 * m[t] + (1.f - b1) * gt;
  const float vt = b2 * v[t] + (1.f - b2) * gt * gt;
  m[t] = mt;
  v[t] = vt;
  p[t] -= lr * (mt / c1) / (sqrtf(vt / c2) + 1e-8f);
}

// normalise features: Z = (X - mean) / std
__global__ void k_normalise(const float* X, const float* mean, const float* sd, float* Z, int n) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) Z[t] = (X[t] - mean[t % NF]) / sd[t % NF];
}

// outputs back to log-milliseconds
__global__ void k_denormalise(float* Y, const float* mean, const float* sd, int n) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) Y[t] = Y[t] * sd[t % NO] + mean[t % NO];
}

inline unsigned blocks(int n) { return (unsigned)((n + 255) / 256); }

// The model: parameters on the host (for save/load) and per device.
struct Model {
  std::mutex mu;
  bool ready = false;
  std::vector<float> host = std::vector<float>(NTOTAL, 0.f);
};
Model g_model;

// device scratch of one forward/backward pass over a mini-batch
struct Net {
  float *p = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
  float *x = nullptr, *h1 = nullptr, *h2 = nullptr, *y = nullptr;
  float *dy = nullptr, *dh2 = nullptr, *dh1 = nullptr, *t = nullptr, *mask = nullptr, *loss = nullptr;
  int cap = 0;
  ~Net() {
    for (float* q : {p, g, m, v, x, h1, h2, y, dy, dh2, dh1, t, mask, loss})
      if (q) cudaFree(q);
  }
  cudaError_t reserve(int B) {
    if (!p) {
      for (float** q : {&p, &g, &m, &v}) {
        if (cudaError_t e = cudaMalloc(q, NTOTAL * sizeof(float))) return e;
      }
      if (cudaError_t e = cudaMalloc(&loss, sizeof(float))) return e;
    }
    if (B <= cap) return cudaSuccess;
    for (float* q : {x, h1, h2, y, dy, dh2, dh1, t, mask})
      if (q) cudaFree(q);
    const size_t f = sizeof(float);
    for (auto pr : {std::make_pair(&x, NF), std::make_pair(&h1, NH), std::make_pair(&h2, NH),
                    std::make_pair(&y, NO), std::make_pair(&dy, NO), std::make_pair(&dh2, NH),
                    std::make_pair(&dh1, NH), std::make_pair(&t, NO), std::make_pair(&mask, NO)}) {
      if (cudaError_t e = cudaMalloc(pr.first, (size_t)B * pr.second * f)) return e;
    }
    cap = B;
    return cudaSuccess;
  }
  void forward(int B, cudaStream_t s) {
    k_dense_fwd<<<blocks(B * NH), 256, 0, s>>>(x, p + OW1, p + OB1, h1, B, NF, NH, 1);
    k_dense_fwd<<<blocks(B * NH), 256, 0, s>>>(h1, p + OW2, p + OB2, h2, B, NH, NH, 1);
    k_dense_fwd<<<blocks(B * NO), 256, 0, s>>>(h2, p + OW3, p + OB3, y, B, NH, NO, 0);
  }
  void backward(int B, cudaStream_t s) {
    k_dense_bwd_w<<<blocks(NH * NO + NO), 256, 0, s>>>(h2, dy, g + OW3, g + OB3, B, NH, NO);
    k_dense_bwd_x<<<blocks(B * NH), 256, 0, s>>>(dy, p + OW3, h2, dh2, B, NH, NO);
    k_dense_bwd_w<<<blocks(NH * NH + NH), 256, 0, s>>>(h1, dh2, g + OW2, g + OB2, B, NH, NH);
    k_dense_bwd_x<<<blocks(B * NH), 256, 0, s>>>(dh2, p + OW2, h1, dh1, B, NH, NH);
    k_dense_bwd_w<<<blocks(NF * NH + NH), 256, 0, s>>>(x, dh1, g + OW1, g + OB1, B, NF, NH);
  }
};

// deterministic initialisation (He-uniform from a 64-bit generator)
void init_params(std::vector<float>& w, uint64_t seed) {
  uint64_t st = seed ^ 0x2545F4914F6CDD1Dull;
  auto next = [&]() {
    st ^= st << 13; st ^= st >> 7; st ^= st << 17;
    return (double)(st >> 11) / 9007199254740992.0;
  };
  auto fill = [&](int off, int fan_in, int count) {
    const double a = std::sqrt(6.0 / fan_in);
    for (int k = 0; k < count; ++k) w[off + k] = (float)((2.0 * next() - 1.0) * a);
  };
  fill(OW1, NF, NF * NH);
  fill(OW2, NH, NH * NH);
  fill(OW3, NH, NH * NO);
  for (int k = 0; k < NH; ++k) { w[OB1 + k] = 0.f; w[OB2 + k] = 0.f; }
  for (int k = 0; k < NO; ++k) w[OB3 + k] = 0.f;
}

}  // namespace

bool cc3dgpu::g_model_loaded() {
  std::lock_guard<std::mutex> lock(g_model.mu);
  return g_model.ready;
}

// ------------------------------------------------------------ C ABI
extern "C" int cc3d_gpu_volume_features(const void* in, int dtype, int64_t sx, int64_t sy, int64_t sz,
                                        int64_t connectivity, int binary_image, int mem_flags, void* stream,
                                        float* features) {
  if (!features || sx <= 0 || sy <= 0 || sz <= 0) return failf(CC3D_ERR_INVALID, "invalid arguments");
  if (!(mem_flags & CC3D_IN_DEVICE) || !device_accessible(in))
    return failf(CC3D_ERR_INVALID, "features need a device volume");
  cudaStream_t s = (cudaStream_t)stream;
  // one small scratch per host thread and device: sums, samples, distinct count
  static thread_local void* scratch = nullptr;
  static thread_local int scratch_dev = -1;
  const size_t bytes = sizeof(FeatureSums) + kDistinct * sizeof(unsigned long long) + 16;
  int dev = 0;
  CKC(cudaGetDevice(&dev));
  if (scratch && scratch_dev != dev) scratch = nullptr;  // kept for the other device's lifetime
  if (!scratch) {
    CKC(cudaMalloc(&scratch, bytes));
    scratch_dev = dev;
  }
  FeatureSums* sums = (FeatureSums*)scratch;
  unsigned long long* samples = (unsigned long long*)((char*)scratch + sizeof(FeatureSums));
  unsigned int* dcount = (unsigned int*)(samples + kDistinct);
  CKC(cudaMemsetAsync(scratch, 0, bytes, s));
  const int64_t voxels = sx * sy * sz;
  const int nsamp = voxels < kDistinct ? (int)voxels : kDistinct;
  switch (dtype) {
    case CC3D_U8: k_features<uint8_t><<<64, 256, 0, s>>>((const uint8_t*)in, sx, sy, sz, sums, samples); break;
    case CC3D_U16: k_features<uint16_t><<<64, 256, 0, s>>>((const uint16_t*)in, sx, sy, sz, sums, samples); break;
    case CC3D_U32: case CC3D_F32:
      k_features<uint32_t><<<64, 256, 0, s>>>((const uint32_t*)in, sx, sy, sz, sums, samples); break;
    case CC3D_U64: case CC3D_F64:
      k_features<uint64_t><<<64, 256, 0, s>>>((const uint64_t*)in, sx, sy, sz, sums, samples); break;
    default: return failf(CC3D_ERR_INVALID, "unknown dtype code %d", dtype);
  }
  k_distinct<<<1, 1024, 0, s>>>(samples, nsamp, dcount);
  CKC(cudaGetLastError());
  FeatureSums h;
  unsigned int distinct = 0;
  CKC(cudaMemcpyAsync(&h, sums, sizeof(h), cudaMemcpyDeviceToHost, s));
  CKC(cudaMemcpyAsync(&distinct, dcount, sizeof(distinct), cudaMemcpyDeviceToHost, s));
  CKC(cudaStreamSynchronize(s));
  const double nsamples = (double)kSamples;
  const double fgf = h.fg / nsamples;
  auto rate = [](unsigned long long a, unsigned long long b) { return b ? (double)a / (double)b : 0.0; };
  auto waste = [](int64_t n, int64_t t) { return 1.0 - (double)n / (double)(t * ((n + t - 1) / t)); };
  const int isz = (dtype == CC3D_U8) ? 1 : (dtype == CC3D_U16) ? 2 : (dtype == CC3D_U32 || dtype == CC3D_F32) ? 4 : 8;
  float f[NF] = {
      (float)std::log2((double)sx), (float)std::log2((double)sy), (float)std::log2((double)sz),
      (float)std::log2((double)voxels), (float)isz / 8.f, (float)connectivity / 26.f, binary_image ? 1.f : 0.f,
      (float)fgf, (float)(std::log2(1.0 + distinct) / 12.0), (float)rate(h.same_x, h.valid_x),
      (float)rate(h.same_y, h.valid_y), (float)rate(h.same_z, h.valid_z), (float)waste(sx, 32),
      (float)waste(sy, 8), (float)waste(sz, 8), (float)rate(h.start_x, h.fg)};
  memcpy(features, f, sizeof(f));
  return CC3D_OK;
}

extern "C" int cc3d_gpu_cost_model_set(const float* params, int n) {
  if (!params || n != NTOTAL) return failf(CC3D_ERR_INVALID, "the cost model has %d parameters", NTOTAL);
  std::lock_guard<std::mutex> lock(g_model.mu);
  g_model.host.assign(params, params + n);
  g_model.ready = true;
  return CC3D_OK;
}

extern "C" int cc3d_gpu_cost_model_get(float* params, int n) {
  if (!params || n != NTOTAL) return failf(CC3D_ERR_INVALID, "the cost model has %d parameters", NTOTAL);
  std::lock_guard<std::mutex> lock(g_model.mu);
  if (!g_model.ready) return failf(CC3D_ERR_INVALID, "no cost model has been trained or loaded");
  memcpy(params, g_model.host.data(), NTOTAL * sizeof(float));
  return CC3D_OK;
}

extern "C" int cc3d_gpu_cost_model_train(const float* X, const float* Y, int n, int epochs, int batch,
                                         float lr, uint64_t seed, float* final_loss) {
  if (!X || !Y || n < 2 || epochs < 1) return failf(CC3D_ERR_INVALID, "invalid arguments");
  if (batch < 1) batch = 256;
  if (batch > n) batch = n;
  // normalisation from the data: features, and log-times over measured entries (Y finite)
  std::vector<float> w(NTOTAL, 0.f);
  init_params(w, seed);
  for (int f = 0; f < NF; ++f) {
    double m = 0, q = 0;
    for (int i = 0; i < n; ++i) { m += X[i * NF + f]; q += (double)X[i * NF + f] * X[i * NF + f]; }
    m /= n;
    const double sd = std::sqrt(std::max(q / n - m * m, 1e-12));
    w[OFM + f] = (float)m;
    w[OFS + f] = (float)(sd > 1e-6 ? sd : 1.0);
  }
  for (int o = 0; o < NO; ++o) {
    double m = 0, q = 0;
    int c = 0;
    for (int i = 0; i < n; ++i)
      if (std::isfinite(Y[i * NO + o])) { m += Y[i * NO + o]; q += (double)Y[i * NO + o] * Y[i * NO + o]; ++c; }
    m = c ? m / c : 0.0;
    const double sd = c ? std::sqrt(std::max(q / c - m * m, 1e-12)) : 1.0;
    w[OOM + o] = (float)m;
    w[OOS + o] = (float)(sd > 1e-6 ? sd : 1.0);
  }
  // normalised training set on the host, uploaded batch by batch
  std::vector<float> Xn((size_t)n * NF), Yn((size_t)n * NO), Mn((size_t)n * NO);
  for (int i = 0; i < n; ++i) {
    for (int f = 0; f < NF; ++f) Xn[(size_t)i * NF + f] = (X[i * NF + f] - w[OFM + f]) / w[OFS + f];
    for (int o = 0; o < NO; ++o) {
      const float y = Y[i * NO + o];
      const bool ok = std::isfinite(y);
      Yn[(size_t)i * NO + o] = ok ? (y - w[OOM + o]) / w[OOS + o] : 0.f;
      Mn[(size_t)i * NO + o] = ok ? 1.f : 0.f;
    }
  }
  Net net;
  CKC(net.reserve(batch));
  float *dX = nullptr, *dY = nullptr, *dM = nullptr;
  CKC(cudaMalloc(&dX, Xn.size() * sizeof(float)));
  CKC(cudaMalloc(&dY, Yn.size() * sizeof(float)));
  CKC(cudaMalloc(&dM, Mn.size() * sizeof(float)));
  cudaStream_t s = nullptr;
  CKC(cudaMemcpy(dX, Xn.data(), Xn.size() * sizeof(float), cudaMemcpyHostToDevice));
  CKC(cudaMemcpy(dY, Yn.data(), Yn.size() * sizeof(float), cudaMemcpyHostToDevice));
  CKC(cudaMemcpy(dM, Mn.data(), Mn.size() * sizeof(float), cudaMemcpyHostToDevice));
  CKC(cudaMemcpy(net.p, w.data(), NTOTAL * sizeof(float), cudaMemcpyHostToDevice));
  CKC(cudaMemset(net.m, 0, NTOTAL * sizeof(float)));
  CKC(cudaMemset(net.v, 0, NTOTAL * sizeof(float)));
  // a fixed shuffle per epoch from the seed (batches are contiguous slices of
  // a permuted copy made on the host)
  std::vector<int> perm(n);
  for (int i = 0; i < n; ++i) perm[i] = i;
  uint64_t st = seed * 0x9E3779B97F4A7C15ull + 1;
  auto rnd = [&]() { st ^= st << 13; st ^= st >> 7; st ^= st << 17; return st; };
  std::vector<float> bx((size_t)batch * NF), by((size_t)batch * NO), bm((size_t)batch * NO);
  int step = 0;
  float last = 0.f;
  const float b1 = 0.9f, b2 = 0.999f;
  for (int ep = 0; ep < epochs; ++ep) {
    for (int i = n - 1; i > 0; --i) std::swap(perm[i], perm[rnd() % (uint64_t)(i + 1)]);
    double ep_loss = 0.0;
    for (int b0 = 0; b0 + batch <= n; b0 += batch) {
      for (int k = 0; k < batch; ++k) {
        const int i = perm[b0 + k];
        memcpy(&bx[(size_t)k * NF], &Xn[(size_t)i * NF], NF * sizeof(float));
        memcpy(&by[(size_t)k * NO], &Yn[(size_t)i * NO], NO * sizeof(float));
        memcpy(&bm[(size_t)k * NO], &Mn[(size_t)i * NO], NO * sizeof(float));
      }
      CKC(cudaMemcpyAsync(net.x, bx.data(), bx.size() * sizeof(float), cudaMemcpyHostToDevice, s));
      CKC(cudaMemcpyAsync(net.t, by.data(), by.size() * sizeof(float), cudaMemcpyHostToDevice, s));
      CKC(cudaMemcpyAsync(net.mask, bm.data(), bm.size() * sizeof(float), cudaMemcpyHostToDevice, s));
      CKC(cudaMemsetAsync(net.loss, 0, sizeof(float), s));
      net.forward(batch, s);
      k_loss<<<blocks(batch * NO), 256, 0, s>>>(net.y, net.t, net.mask, net.dy, net.loss, batch * NO);
      net.backward(batch, s);
      ++step;
      const float c1 = 1.f - std::pow(b1, (float)step), c2 = 1.f - std::pow(b2, (float)step);
      k_adam<<<blocks(NPARAM), 256, 0, s>>>(net.p, net.g, net.m, net.v, NPARAM, lr, b1, b2, c1, c2);
      float hl = 0.f;
      CKC(cudaMemcpyAsync(&hl, net.loss, sizeof(float), cudaMemcpyDeviceToHost, s));
      CKC(cudaStreamSynchronize(s));
      ep_loss += hl;
    }
    last = (float)(ep_loss / ((double)(n / batch) * batch));
  }
  CKC(cudaGetLastError());
  CKC(cudaMemcpy(w.data(), net.p, NPARAM * sizeof(float), cudaMemcpyDeviceToHost));
  cudaFree(dX);
  cudaFree(dY);
  cudaFree(dM);
  {
    std::lock_guard<std::mutex> lock(g_model.mu);
    g_model.host = w;
    g_model.ready = true;
  }
  if (final_loss) *final_loss = last;
  return CC3D_OK;
}

extern "C" int cc3d_gpu_cost_model_predict(const float* X, int n, float* Y) {
  if (!X || !Y || n < 1) return failf(CC3D_ERR_INVALID, "invalid arguments");
  std::vector<float> w;
  {
    std::lock_guard<std::mutex> lock(g_model.mu);
    if (!g_model.ready) return failf(CC3D_ERR_INVALID, "no cost model has been trained or loaded");
    w = g_model.host;
  }
  static thread_local Net net;
  static thread_local float* dXraw = nullptr;
  static thread_local int raw_cap = 0;
  CKC(net.reserve(n));
  if (n > raw_cap) {
    if (dXraw) cudaFree(dXraw);
    dXraw = nullptr;
    raw_cap = 0;
    CKC(cudaMalloc(&dXraw, (size_t)n * NF * sizeof(float)));
    raw_cap = n;
  }
  cudaStream_t s = nullptr;
  CKC(cudaMemcpy(net.p, w.data(), NTOTAL * sizeof(float), cudaMemcpyHostToDevice));
  CKC(cudaMemcpy(dXraw, X, (size_t)n * NF * sizeof(float), cudaMemcpyHostToDevice));
  k_normalise<<<blocks(n * NF), 256, 0, s>>>(dXraw, net.p + OFM, net.p + OFS, net.x, n * NF);
  net.forward(n, s);
  k_denormalise<<<blocks(n * NO), 256, 0, s>>>(net.y, net.p + OOM, net.p + OOS, n * NO);
  CKC(cudaGetLastError());
  CKC(cudaMemcpy(Y, net.y, (size_t)n * NO * sizeof(float), cudaMemcpyDeviceToHost));
  return CC3D_OK;
}

extern "C" int cc3d_gpu_cost_model_choose(const void* in, int dtype, int64_t sx, int64_t sy, int64_t sz,
                                          int64_t connectivity, int binary_image, int mem_flags, void* stream,
                                          float min_margin, int* choice, int* confident) {
  if (!choice || !confident) return failf(CC3D_ERR_INVALID, "invalid arguments");
  const int conn = (int)connectivity;
  if (binary_image && conn == 8) {  // one configuration only (2x2-block numbering)
    *choice = CC3D_TILE_RUNS;
    *confident = 1;
    return CC3D_OK;
  }
  const bool d3 = sz != 1 && (conn == 26 || conn == 18 || conn == 6);
  const int ncfg = d3 ? NO : 4;  // 2D: the 8x8 entries (one tile shape)
  float f[NF], y[NO];
  if (int rc = cc3d_gpu_volume_features(in, dtype, sx, sy, sz, connectivity, binary_image, mem_flags, stream, f))
    return rc;
  if (int rc = cc3d_gpu_cost_model_predict(f, 1, y)) return rc;
  int best = 0;
  for (int k = 1; k < ncfg; ++k)
    if (y[k] < y[best]) best = k;
  float second = INFINITY;
  for (int k = 0; k < ncfg; ++k)
    if (k != best && y[k] < second) second = y[k];
  if (second - y[best] >= std::log1p(min_margin)) {
    *choice = cc3d_gpu_tile_config(best);
    *confident = 1;
    return CC3D_OK;
  }
  *confident = 0;  // too close to call: time them all
  return cc3d_gpu_autotune(in, dtype, sx, sy, sz, connectivity, binary_image, mem_flags, stream, 1, choice,
                           nullptr);
}
