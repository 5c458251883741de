// Autotuner and learned cost model (no counterpart in the reference, whose
// plan is fixed at compile time by its factor list, src/gfftfactor.h).
//
//  - gfft_tune_candidates: the distinct plans reachable through the plan
//    options (radix order, largest radix, kernel variant, pipeline depth,
//    pass-length cap), de-duplicated by their resulting pass structure;
//  - gfft_tune_measure: times every candidate on caller-provided device
//    buffers with CUDA events (exhaustive measured search);
//  - gfft_plan_features: the feature vector of a plan for the cost model;
//  - gfft_mlp_*: a small multi-layer perceptron (FP32, hidden layers of
//    equal width, ReLU) trained on the GPU by the kernels below: a forward
//    kernel (one thread per sample, weights in shared memory), a backward
//    kernel that recomputes the forward pass, back-propagates the squared
//    error and sums the per-sample gradients (shared-memory atomics, then one
//    global atomic per parameter and block), and an Adam update kernel.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/gfft_gb300.h"
#include "plan.h"

// ---------------------------------------------------------------- tuner ----
namespace {

bool same_plan(const gfft_plan_info& a, const gfft_plan_info& b) {
  if (a.n_global_passes != b.n_global_passes) return false;
  for (int g = 0; g < a.n_global_passes; ++g) {
    if (a.pass_len[g] != b.pass_len[g] || a.threads[g] != b.threads[g] || a.units[g] != b.units[g] ||
        a.kernel_variant[g] != b.kernel_variant[g])
      return false;
    for (int i = 0; i < 16; ++i)
      if (a.radices[g][i] != b.radices[g][i]) return false;
  }
  return true;
}

}  // namespace

extern "C" {

int gfft_tune_candidates(uint64_t n, int vtype_id, int trans_id, int place_id, uint64_t batch,
                         gfft_plan_opts* cands, int max_cands, int* ncands) {
  if (!cands || !ncands) return GFFT_E_NULL_POINTER;
  *ncands = 0;
  std::vector<gfft_plan_info> seen;
  // structural knobs; pipeline depths are varied only around the default
  const int orders[] = {0, 1, 2};
  const int radices[] = {16, 8, 4};
  const int variants[] = {0, 1};
  const int caps[] = {0, 4096, 1024, 256, 64};
  struct K {
    int cap, v, mr, ro, st, w, bps = 0;
  };
  std::vector<K> ks;
  // pipeline depths other than the default (one stage FP32, two FP64)
  const int dflt_st = (vtype_id == 0 || vtype_id == 2) ? 2 : 1;
  ks.push_back({0, 0, 16, 0, 0, 0});
  for (int st : {1, 2, 3})
    if (st != dflt_st) ks.push_back({0, 0, 16, 0, st, 0});
  // 64 KB tensor-copy tiles where FP32 passes of 128 .. 512 default to 32 KB,
  // and 32 KB tiles on FP32 passes of 1024 too
  for (int cap : {0, 4096, 1024}) ks.push_back({cap, 0, 16, 0, 0, 0, 1});
  for (int cap : {0, 4096}) ks.push_back({cap, 0, 16, 0, 0, 0, 2});
  // wider column tiles (128- and 256-byte rows) with shorter passes
  for (int cap : {0, 512, 256, 128})
    for (int w : {16, 32}) ks.push_back({cap, 0, 16, 0, 0, w});
  // the prefetching and the specialised column tiles where the tensor-copy
  // ones are the default
  for (int cap : caps) ks.push_back({cap, 4, 16, 0, 0, 0});
  for (int cap : caps) ks.push_back({cap, 5, 16, 0, 0, 0});
  // the copy-free mixed-radix tiles where the column tiles of variant 9 take mixed shapes
  for (int cap : caps) ks.push_back({cap, 7, 16, 0, 0, 0});
  for (int cap : caps)
    for (int v : variants)
      for (int mr : radices)
        for (int ro : orders) ks.push_back({cap, v, mr, ro, 0, 0});
  for (const K& k : ks) {
    gfft_plan_opts o;
    std::memset(&o, 0, sizeof(o));
    o.radix_order = k.ro;
    o.max_radix = k.mr == 16 ? 0 : k.mr;
    o.kernel_variant = k.v;
    o.stages = k.st;
    o.max_pass_len = k.cap;
    o.units_per_block = k.w;
    o.blocks_per_sm = k.bps;
    gfft_plan_info info;
    if (gfft_plan_query(n, vtype_id, trans_id, place_id, batch, &o, &info) != GFFT_OK) continue;
    if (k.w != 0) {  // a lane width only where the column-tile kernel runs
      bool lanes = false;
      for (int g = 0; g < info.n_global_passes; ++g) lanes |= (info.kernel_variant[g] == 4);
      if (!lanes) continue;
    }
    if (k.st != 0) {  // a depth variant only where a pipelined kernel runs
      bool pipelined = false;
      for (int g = 0; g < info.n_global_passes; ++g)
        pipelined |= (info.kernel_variant[g] == 2 || info.kernel_variant[g] == 3 || info.kernel_variant[g] == 9);
      if (!pipelined) continue;
    } else {
      bool dup = false;
      for (const gfft_plan_info& s : seen) dup |= same_plan(s, info);
      if (dup) continue;
      seen.push_back(info);
    }
    if (*ncands >= max_cands) return GFFT_OK;
    cands[(*ncands)++] = o;
  }
  return GFFT_OK;
}

int gfft_tune_measure(uint64_t n, int vtype_id, int trans_id, int place_id, uint64_t batch,
                      const gfft_plan_opts* cands, int ncands, const void* d_src, void* d_dst, int reps,
                      float* ms_out) {
  if (!cands || !ms_out || !d_src || !d_dst) return GFFT_E_NULL_POINTER;
  if (reps < 1) reps = 1;
  cudaStream_t s;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return GFFT_E_CUDA;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int status = GFFT_OK;
  for (int c = 0; c < ncands; ++c) {
    ms_out[c] = -1.0f;
    gfft_handle h = nullptr;
    if (gfft_create_opts(&h, n, vtype_id, trans_id, 1, 0, place_id, batch, &cands[c]) != GFFT_OK) continue;
    const void* src = place_id == 0 ? d_dst : d_src;
    int st = gfft_exec(h, src, d_dst, (gfft_stream)s);  // warm-up
    if (st == GFFT_OK) {
      cudaEventRecord(e0, s);
      for (int r = 0; r < reps && st == GFFT_OK; ++r) st = gfft_exec(h, src, d_dst, (gfft_stream)s);
      cudaEventRecord(e1, s);
      cudaEventSynchronize(e1);
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      if (st == GFFT_OK) ms_out[c] = ms / reps;
    }
    if (st != GFFT_OK) status = st;
    gfft_destroy(h);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(s);
  return status == GFFT_E_CUDA ? status : GFFT_OK;
}

int gfft_plan_features(uint64_t n, int vtype_id, int trans_id, int place_id, uint64_t batch,
                       const gfft_plan_opts* opts, float* f) {
  if (!f) return GFFT_E_NULL_POINTER;
  gfft_plan_info info;
  int st = gfft_plan_query(n, vtype_id, trans_id, place_id, batch, opts, &info);
  if (st != GFFT_OK) return st;
  std::memset(f, 0, sizeof(float) * GFFT_NFEAT);
  uint64_t m = n;
  int e[4] = {0, 0, 0, 0};
  const uint64_t pr[4] = {2, 3, 5, 7};
  for (int i = 0; i < 4; ++i)
    while (m % pr[i] == 0) {
      m /= pr[i];
      ++e[i];
    }
  const int dbl = (vtype_id == 0 || vtype_id == 2) ? 1 : 0;
  f[0] = (float)std::log2((double)n);
  for (int i = 0; i < 4; ++i) f[1 + i] = (float)e[i];
  f[5] = (float)std::log2((double)batch);
  f[6] = (float)dbl;
  f[7] = (float)info.n_global_passes;
  const int rlist[7] = {16, 8, 4, 2, 3, 5, 7};
  double lw = 0.0;
  int lmax = 0, lmin = 1 << 30;
  for (int g = 0; g < info.n_global_passes; ++g) {
    for (int i = 0; i < 16 && info.radices[g][i]; ++i)
      for (int k = 0; k < 7; ++k)
        if (info.radices[g][i] == rlist[k]) f[8 + k] += 1.0f;
    lw += std::log2((double)std::max(1, info.units[g]));
    lmax = std::max(lmax, info.pass_len[g]);
    lmin = std::min(lmin, info.pass_len[g]);
    const int v = info.kernel_variant[g];
    f[v <= 1 ? 18 : (v <= 3 ? 19 : (v == 4 ? 20 : (v == 9 ? 24 : 21)))] += 1.0f;
  }
  f[15] = (float)(lw / std::max(1, info.n_global_passes));  // mean log2 units (transforms or lanes per block)
  f[16] = (float)std::log2((double)std::max(1, lmax));
  f[17] = (float)std::log2((double)std::max(1, lmin));
  f[22] = opts ? (float)opts->stages : 0.0f;
  f[23] = (float)info.radices[0][0] / 16.0f;  // the first radix (radix order)
  return GFFT_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ MLP ----
namespace mlp {

constexpr int MAXW = 64;     // widest layer
constexpr int MAXL = 4;      // hidden layers
constexpr int MAXIN = 32;    // inputs

struct Shape {
  int nin, width, depth;     // depth hidden layers of `width`, then one output
  int off_w[MAXL + 1], off_b[MAXL + 1], in_of[MAXL + 1], out_of[MAXL + 1];
  int nparams;
};

Shape make_shape(int nin, int width, int depth) {
  Shape s;
  s.nin = nin;
  s.width = width;
  s.depth = depth;
  int off = 0;
  for (int l = 0; l <= depth; ++l) {
    s.in_of[l] = l == 0 ? nin : width;
    s.out_of[l] = l == depth ? 1 : width;
    s.off_w[l] = off;
    off += s.in_of[l] * s.out_of[l];
    s.off_b[l] = off;
    off += s.out_of[l];
  }
  s.nparams = off;
  return s;
}

// forward of one sample with weights in shared memory; acts[l][k] kept for
// the backward pass (post-ReLU values of hidden layer l)
__device__ float forward_one(const Shape& s, const float* P, const float* x, float acts[MAXL][MAXW]) {
  float in[MAXW];
  for (int i = 0; i < s.nin; ++i) in[i] = x[i];
  float out = 0.f;
  for (int l = 0; l <= s.depth; ++l) {
    const float* Wl = P + s.off_w[l];
    const float* bl = P + s.off_b[l];
    const int ni = s.in_of[l], no = s.out_of[l];
    if (l == s.depth) {
      float acc = bl[0];
      for (int i = 0; i < ni; ++i) acc = fmaf(Wl[i], in[i], acc);
      out = acc;
    } else {
      for (int o = 0; o < no; ++o) {
        float acc = bl[o];
        for (int i = 0; i < ni; ++i) acc = fmaf(Wl[o * ni + i], in[i], acc);
        acts[l][o] = acc > 0.f ? acc : 0.f;
      }
      for (int o = 0; o < no; ++o) in[o] = acts[l][o];
    }
  }
  return out;
}

__global__ void forward_kernel(const Shape s, const float* __restrict__ params, const float* __restrict__ X, int n,
                               float* __restrict__ y) {
  extern __shared__ float P[];
  for (int i = threadIdx.x; i < s.nparams; i += blockDim.x) P[i] = params[i];
  __syncthreads();
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    float acts[MAXL][MAXW];
    y[k] = forward_one(s, P, X + (long long)k * s.nin, acts);
  }
}

// gradients of L = (1/n) sum_k (f(x_k) - t_k)^2, summed into grad (zeroed by
// the caller); loss_sum += sum_k (f - t)^2
__global__ void backward_kernel(const Shape s, const float* __restrict__ params, const float* __restrict__ X,
                                const float* __restrict__ t, int n, float* __restrict__ grad, float* loss_sum) {
  extern __shared__ float sh[];
  float* P = sh;
  float* G = sh + s.nparams;
  for (int i = threadIdx.x; i < s.nparams; i += blockDim.x) {
    P[i] = params[i];
    G[i] = 0.f;
  }
  __syncthreads();
  float lsum = 0.f;
  const float inv_n = 1.0f / (float)n;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const float* x = X + (long long)k * s.nin;
    float acts[MAXL][MAXW];
    const float f = forward_one(s, P, x, acts);
    const float r = f - t[k];
    lsum += r * r;
    // delta of the output layer
    float delta[MAXW];
    float nd[MAXW];
    delta[0] = 2.f * r * inv_n;
    for (int l = s.depth; l >= 0; --l) {
      const int ni = s.in_of[l], no = s.out_of[l];
      const float* Wl = P + s.off_w[l];
      float* gW = G + s.off_w[l];
      float* gb = G + s.off_b[l];
      const float* a_in = l == 0 ? x : acts[l - 1];
      for (int o = 0; o < no; ++o) {
        atomicAdd(&gb[o], delta[o]);
        for (int i = 0; i < ni; ++i) atomicAdd(&gW[o * ni + i], delta[o] * a_in[i]);
      }
      if (l > 0) {
        for (int i = 0; i < ni; ++i) {
          float acc = 0.f;
          for (int o = 0; o < no; ++o) acc = fmaf(Wl[o * ni + i], delta[o], acc);
          nd[i] = acts[l - 1][i] > 0.f ? acc : 0.f;  // ReLU'
        }
        for (int i = 0; i < ni; ++i) delta[i] = nd[i];
      }
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < s.nparams; i += blockDim.x) atomicAdd(&grad[i], G[i]);
  // block reduction of the loss
  for (int o = 16; o > 0; o >>= 1) lsum += __shfl_down_sync(0xffffffffu, lsum, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss_sum, lsum);
}

__global__ void adam_kernel(float* p, const float* g, float* m, float* v, int np, float lr, float b1, float b2,
                            float eps, float c1, float c2) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

}  // namespace mlp

struct gfft_mlp {
  mlp::Shape shape;
  float* d_params = nullptr;
  float* d_grad = nullptr;
  float* d_m = nullptr;
  float* d_v = nullptr;
  float* d_loss = nullptr;
  long long step = 0;
};

extern "C" {

int gfft_mlp_create(gfft_mlp** out, int nin, int width, int depth, uint64_t seed) {
  if (!out) return GFFT_E_NULL_POINTER;
  *out = nullptr;
  if (nin < 1 || nin > mlp::MAXIN || width < 1 || width > mlp::MAXW || depth < 1 || depth > mlp::MAXL)
    return GFFT_E_INVALID_SIZE;
  gfft_mlp* m = new (std::nothrow) gfft_mlp();
  if (!m) return GFFT_E_ALLOC;
  m->shape = mlp::make_shape(nin, width, depth);
  const int np = m->shape.nparams;
  // He initialisation from a splitmix64 stream (Box-Muller), zero biases
  std::vector<float> p(np, 0.f);
  uint64_t s = seed;
  auto next = [&]() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return ((z ^ (z >> 31)) >> 11) * (1.0 / 9007199254740992.0);
  };
  for (int l = 0; l <= depth; ++l) {
    const double sd = std::sqrt(2.0 / m->shape.in_of[l]);
    for (int i = 0; i < m->shape.in_of[l] * m->shape.out_of[l]; ++i) {
      double u1 = next() + 1e-300, u2 = next();
      p[m->shape.off_w[l] + i] = (float)(sd * std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2));
    }
  }
  const size_t b = (size_t)np * sizeof(float);
  if (cudaMalloc(&m->d_params, b) != cudaSuccess || cudaMalloc(&m->d_grad, b) != cudaSuccess ||
      cudaMalloc(&m->d_m, b) != cudaSuccess || cudaMalloc(&m->d_v, b) != cudaSuccess ||
      cudaMalloc(&m->d_loss, sizeof(float)) != cudaSuccess) {
    cudaFree(m->d_params);
    cudaFree(m->d_grad);
    cudaFree(m->d_m);
    cudaFree(m->d_v);
    delete m;
    return GFFT_E_ALLOC;
  }
  cudaMemcpy(m->d_params, p.data(), b, cudaMemcpyHostToDevice);
  cudaMemset(m->d_m, 0, b);
  cudaMemset(m->d_v, 0, b);
  *out = m;
  return GFFT_OK;
}

int gfft_mlp_num_params(gfft_mlp* m) { return m ? m->shape.nparams : -1; }

int gfft_mlp_get_params(gfft_mlp* m, float* p) {
  if (!m || !p) return GFFT_E_NULL_POINTER;
  return cudaMemcpy(p, m->d_params, (size_t)m->shape.nparams * sizeof(float), cudaMemcpyDeviceToHost) == cudaSuccess
             ? GFFT_OK
             : GFFT_E_CUDA;
}

int gfft_mlp_set_params(gfft_mlp* m, const float* p) {
  if (!m || !p) return GFFT_E_NULL_POINTER;
  return cudaMemcpy(m->d_params, p, (size_t)m->shape.nparams * sizeof(float), cudaMemcpyHostToDevice) == cudaSuccess
             ? GFFT_OK
             : GFFT_E_CUDA;
}

static int upload_xy(const float* X, const float* y, int n, int nin, float** dX, float** dy) {
  *dX = nullptr;
  *dy = nullptr;
  if (cudaMalloc(dX, (size_t)n * nin * sizeof(float)) != cudaSuccess) return GFFT_E_ALLOC;
  if (cudaMemcpy(*dX, X, (size_t)n * nin * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) return GFFT_E_CUDA;
  if (y) {
    if (cudaMalloc(dy, (size_t)n * sizeof(float)) != cudaSuccess) return GFFT_E_ALLOC;
    if (cudaMemcpy(*dy, y, (size_t)n * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) return GFFT_E_CUDA;
  }
  return GFFT_OK;
}

static int backward_launch(gfft_mlp* m, const float* dX, const float* dy, int n) {
  const int np = m->shape.nparams;
  cudaMemset(m->d_grad, 0, (size_t)np * sizeof(float));
  cudaMemset(m->d_loss, 0, sizeof(float));
  const size_t smem = 2 * (size_t)np * sizeof(float);
  cudaFuncSetAttribute(mlp::backward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const int threads = 128;
  const int blocks = std::max(1, std::min(64, (n + threads - 1) / threads));
  mlp::backward_kernel<<<blocks, threads, smem>>>(m->shape, m->d_params, dX, dy, n, m->d_grad, m->d_loss);
  return cudaGetLastError() == cudaSuccess ? GFFT_OK : GFFT_E_CUDA;
}

// gradients (summed over the samples, loss = mean squared error) for the
// gradient check against the CPU reference
int gfft_mlp_gradients(gfft_mlp* m, const float* X, const float* y, int n, float* grad_out, float* loss_out) {
  if (!m || !X || !y || !grad_out) return GFFT_E_NULL_POINTER;
  float *dX, *dy;
  int st = upload_xy(X, y, n, m->shape.nin, &dX, &dy);
  if (st == GFFT_OK) st = backward_launch(m, dX, dy, n);
  if (st == GFFT_OK &&
      cudaMemcpy(grad_out, m->d_grad, (size_t)m->shape.nparams * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
    st = GFFT_E_CUDA;
  if (st == GFFT_OK && loss_out) {
    float l;
    cudaMemcpy(&l, m->d_loss, sizeof(float), cudaMemcpyDeviceToHost);
    *loss_out = l / (float)n;
  }
  cudaFree(dX);
  cudaFree(dy);
  return st;
}

// full-batch Adam on the GPU; *final_loss = the mean squared error of the last epoch
int gfft_mlp_train(gfft_mlp* m, const float* X, const float* y, int n, int epochs, float lr, float* final_loss) {
  if (!m || !X || !y) return GFFT_E_NULL_POINTER;
  if (n < 1 || epochs < 1) return GFFT_E_INVALID_SIZE;
  float *dX, *dy;
  int st = upload_xy(X, y, n, m->shape.nin, &dX, &dy);
  const int np = m->shape.nparams;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (int e = 0; e < epochs && st == GFFT_OK; ++e) {
    st = backward_launch(m, dX, dy, n);
    ++m->step;
    const float c1 = 1.f - std::pow(b1, (float)m->step), c2 = 1.f - std::pow(b2, (float)m->step);
    mlp::adam_kernel<<<(np + 255) / 256, 256>>>(m->d_params, m->d_grad, m->d_m, m->d_v, np, lr, b1, b2, eps, c1, c2);
    if (cudaGetLastError() != cudaSuccess) st = GFFT_E_CUDA;
  }
  if (st == GFFT_OK && final_loss) {
    float l;
    cudaMemcpy(&l, m->d_loss, sizeof(float), cudaMemcpyDeviceToHost);
    *final_loss = l / (float)n;
  }
  cudaFree(dX);
  cudaFree(dy);
  return st;
}

int gfft_mlp_predict(gfft_mlp* m, const float* X, int n, float* y_out) {
  if (!m || !X || !y_out) return GFFT_E_NULL_POINTER;
  float *dX, *dy;
  int st = upload_xy(X, nullptr, n, m->shape.nin, &dX, &dy);
  if (st == GFFT_OK && cudaMalloc(&dy, (size_t)n * sizeof(float)) != cudaSuccess) st = GFFT_E_ALLOC;
  if (st == GFFT_OK) {
    const size_t smem = (size_t)m->shape.nparams * sizeof(float);
    cudaFuncSetAttribute(mlp::forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    mlp::forward_kernel<<<std::max(1, std::min(64, (n + 127) / 128)), 128, smem>>>(m->shape, m->d_params, dX, n, dy);
    if (cudaGetLastError() != cudaSuccess) st = GFFT_E_CUDA;
  }
  if (st == GFFT_OK && cudaMemcpy(y_out, dy, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
    st = GFFT_E_CUDA;
  cudaFree(dX);
  cudaFree(dy);
  return st;
}

int gfft_mlp_destroy(gfft_mlp* m) {
  if (!m) return GFFT_E_INVALID_HANDLE;
  cudaFree(m->d_params);
  cudaFree(m->d_grad);
  cudaFree(m->d_m);
  cudaFree(m->d_v);
  cudaFree(m->d_loss);
  delete m;
  return GFFT_OK;
}

}  // extern "C"
