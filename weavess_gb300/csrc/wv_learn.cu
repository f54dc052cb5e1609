// Learned entry point and beam width for the greedy search (not in the
// reference: an addition beside the plain form, with the plain search as its
// fallback and as the judge of its recall).
//
//  * clusters: k-means (Lloyd) on the base; each cluster keeps an entry list,
//    its member nearest the centroid followed by further members, used as the
//    search seeds of a query routed to it;
//  * traces: the plain search (random entry, beam L_trace) answers every
//    training query; the cluster of its first result is the entry label, and
//    the smallest beam (from a grid) whose answer, started from that
//    cluster's list, matches the plain answer in >= 9 of 10 ids is the
//    beam label (as log2 L);
//  * model: x -> 256 -> 256 (ReLU) -> C entry logits + 1 beam regressor, BF16
//    operands with FP32 accumulation in tensor memory (tcgen05, wv_umma.cu),
//    softmax cross-entropy + squared error, Adam; every forward, backward and
//    update step is a kernel of this file;
//  * inference: one forward pass per query batch picks the entry cluster(s)
//    and the beam width, writes seeds and per-query L, and runs the batched
//    search (mixed L in one launch).  Queries the model is unsure of
//    (top-1 probability below `fallback_p`) take the plain search (random
//    seeds, beam L_plain).
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "wv_common.cuh"
#include "wv_ctx.h"
#include "wv_learn.h"
#include "wv_mlp.cuh"
#include "wv_search.h"
#include "wv_seeds.h"

namespace wv {
namespace {

constexpr uint32_t HID = 256;

// ---------------------------------------------------------------- k-means
// warp per point: nearest of C centroids (in shared memory)
__global__ void k_km_assign(const float *x, uint32_t n, uint32_t d, const float *cent, uint32_t C, uint32_t *asg,
                            float *dist) {
  extern __shared__ float sc[];  // C rows of d + 1 floats (padded: lanes read different rows)
  for (uint32_t i = threadIdx.x; i < C * d; i += blockDim.x) sc[(i / d) * (d + 1) + i % d] = cent[i];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t p = w; p < n; p += nw) {
    const float *row = x + (size_t)p * d;
    float best = 3.4e38f;
    uint32_t bi = 0;
    for (uint32_t c = lane; c < C; c += 32) {
      float acc = 0.f;
      for (uint32_t k = 0; k < d; k++) {
        const float e = row[k] - sc[c * (d + 1) + k];
        acc += e * e;
      }
      if (acc < best) {
        best = acc;
        bi = c;
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const float ob = __shfl_xor_sync(FULL, best, o);
      const uint32_t oi = __shfl_xor_sync(FULL, bi, o);
      if (ob < best || (ob == best && oi < bi)) {
        best = ob;
        bi = oi;
      }
    }
    if (lane == 0) {
      asg[p] = bi;
      if (dist) dist[p] = best;
    }
  }
}

__global__ void k_km_accum(const float *x, uint32_t n, uint32_t d, const uint32_t *asg, float *sum, uint32_t *cnt) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= (size_t)n * d) return;
  const uint32_t p = (uint32_t)(i / d), k = (uint32_t)(i % d);
  atomicAdd(&sum[(size_t)asg[p] * d + k], x[i]);
  if (k == 0) atomicAdd(&cnt[asg[p]], 1u);
}

// ---------------------------------------------------------------- MLP kernels
__global__ void k_gather_norm(const float *x, const uint32_t *rows, uint32_t B, uint32_t d, const float *mu,
                              const float *sg, __nv_bfloat16 *out) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= (size_t)B * d) return;
  const uint32_t b = (uint32_t)(i / d), k = (uint32_t)(i % d);
  const uint32_t r = rows ? rows[b] : b;
  out[i] = __float2bfloat16_rn((x[(size_t)r * d + k] - mu[k]) / sg[k]);
}

// softmax cross-entropy on O[:, :C] and squared error on O[:, C];
// dO = d(mean loss) / dO; loss sums into loss[0] (ce) and loss[1] (mse)
__global__ void k_loss_grad(const float *O, uint32_t B, uint32_t C, const uint32_t *yc, const float *yr,
                            const uint32_t *rows, float lam, float *dO, __nv_bfloat16 *dOb, float *loss) {
  const int lane = threadIdx.x & 31;
  const uint32_t b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (b >= B) return;
  const uint32_t r = rows ? rows[b] : b;
  const uint32_t W = C + 1;
  const float *o = O + (size_t)b * W;
  float m = -3.4e38f;
  for (uint32_t c = lane; c < C; c += 32) m = fmaxf(m, o[c]);
  for (int s = 16; s > 0; s >>= 1) m = fmaxf(m, __shfl_xor_sync(FULL, m, s));
  float se = 0.f;
  for (uint32_t c = lane; c < C; c += 32) se += expf(o[c] - m);
  for (int s = 16; s > 0; s >>= 1) se += __shfl_xor_sync(FULL, se, s);
  const uint32_t y = yc[r];
  for (uint32_t c = lane; c < C; c += 32) {
    const float p = expf(o[c] - m) / se;
    const float g = (p - (c == y ? 1.f : 0.f)) / (float)B;
    dO[(size_t)b * W + c] = g;
    dOb[(size_t)b * W + c] = __float2bfloat16_rn(g);
  }
  if (lane == 0) {
    const float e = o[C] - yr[r];
    const float g = 2.f * lam * e / (float)B;
    dO[(size_t)b * W + C] = g;
    dOb[(size_t)b * W + C] = __float2bfloat16_rn(g);
    atomicAdd(&loss[0], (logf(se) + m - o[y]) / (float)B);
    atomicAdd(&loss[1], e * e / (float)B);
  }
}

// dZ = dH * (H > 0), as FP32 and BF16
__global__ void k_relu_bwd(const float *dH, const float *H, size_t count, float *dZ, __nv_bfloat16 *dZb) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float v = H[i] > 0.f ? dH[i] : 0.f;
  dZ[i] = v;
  dZb[i] = __float2bfloat16_rn(v);
}

// db[n] = sum_b dY[b, n]
__global__ void k_colsum(const float *dY, uint32_t B, uint32_t N, float *db) {
  const uint32_t nidx = blockIdx.x * blockDim.x + threadIdx.x;
  if (nidx >= N) return;
  float s = 0.f;
  for (uint32_t b = 0; b < B; b++) s += dY[(size_t)b * N + nidx];
  db[nidx] = s;
}

__global__ void k_adam(float *p, const float *g, float *m, float *v, size_t count, float lr, float b1, float b2,
                       float eps, float c1, float c2) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// out (cols x rows) = x (rows x cols)^T, rounded to bf16
__global__ void k_transpose_bf16(const float *x, uint32_t rows, uint32_t cols, __nv_bfloat16 *out) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= (size_t)rows * cols) return;
  const uint32_t r = (uint32_t)(i / cols), cc = (uint32_t)(i % cols);
  out[(size_t)cc * rows + r] = __float2bfloat16_rn(x[i]);
}

__global__ void k_to_bf16(const float *x, size_t count, __nv_bfloat16 *out) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < count) out[i] = __float2bfloat16_rn(x[i]);
}

// per query: entry cluster(s), beam width and seeds from the model output
__global__ void k_learn_seeds(const float *O, uint32_t nq, uint32_t C, const uint32_t *lists, uint32_t SL,
                              const uint32_t *llen, float margin, uint32_t Lmin, uint32_t Lmax, float fallback_p,
                              uint32_t L_plain, const uint32_t *plain_seeds, uint32_t *seeds, uint32_t stride,
                              uint32_t *Lq, uint32_t K, uint32_t *used_fallback) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  const float *o = O + (size_t)q * (C + 1);
  uint32_t c1 = 0, c2 = 0;
  float v1 = -3.4e38f, v2 = -3.4e38f;
  for (uint32_t c = 0; c < C; c++) {
    const float v = o[c];
    if (v > v1) {
      v2 = v1;
      c2 = c1;
      v1 = v;
      c1 = c;
    } else if (v > v2) {
      v2 = v;
      c2 = c;
    }
  }
  float se = 0.f;
  for (uint32_t c = 0; c < C; c++) se += expf(o[c] - v1);
  const float p1 = 1.f / se;
  uint32_t *sq = seeds + (size_t)q * stride;
  if (plain_seeds && p1 < fallback_p) {  // the plain search
    for (uint32_t j = 0; j < L_plain; j++) sq[j] = plain_seeds[(size_t)q * L_plain + j];
    Lq[q] = L_plain;
    atomicAdd(used_fallback, 1u);
    return;
  }
  float lf = exp2f(o[C]) * margin;
  uint32_t L = (uint32_t)ceilf(lf);
  L = max(Lmin, min(Lmax, max(L, K)));
  Lq[q] = L;
  // seeds: the first cluster's list; when the second cluster is close in
  // probability (p2 > p1 / 4), alternate between the two lists
  const bool two = (expf(v2 - v1) > 0.25f) && llen[c2] > 0;
  uint32_t a = 0, b = 0, t = 0;
  while (t < L) {
    const bool from1 = !two || (t & 1) == 0 || b >= llen[c2];
    if (from1 && a < llen[c1]) sq[t++] = lists[(size_t)c1 * SL + a++];
    else if (two && b < llen[c2]) sq[t++] = lists[(size_t)c2 * SL + b++];
    else break;
  }
  // short lists: fill with the plain seeds not already taken
  for (uint32_t j = 0; plain_seeds && t < L && j < L_plain; j++) {
    const uint32_t id = plain_seeds[(size_t)q * L_plain + j];
    bool dup = false;
    for (uint32_t u = 0; u < t && !dup; u++) dup = sq[u] == id;
    if (!dup) sq[t++] = id;
  }
  Lq[q] = t;
}

// seeds of the label cluster at a fixed beam (trace labelling)
__global__ void k_cluster_seeds(const uint32_t *label, uint32_t nq, const uint32_t *lists, uint32_t SL,
                                const uint32_t *llen, uint32_t L, const uint32_t *plain_seeds, uint32_t Lp,
                                uint32_t *seeds) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  const uint32_t c = label[q];
  uint32_t *sq = seeds + (size_t)q * L;
  uint32_t t = 0;
  for (; t < L && t < llen[c]; t++) sq[t] = lists[(size_t)c * SL + t];
  for (uint32_t j = 0; t < L && j < Lp; j++) {
    const uint32_t id = plain_seeds[(size_t)q * Lp + j];
    bool dup = false;
    for (uint32_t u = 0; u < t && !dup; u++) dup = sq[u] == id;
    if (!dup) sq[t++] = id;
  }
}

}  // namespace

// ================================================================ state
struct LearnState {
  uint32_t C = 0, D = 0, SL = 0;
  std::vector<uint32_t> h_assign;  // k-means cluster of every base row
  // parameter block (FP32 master): W1 D x H, b1 H, W2 H x H, b2 H, W3 H x (C+1), b3 C+1
  size_t oW1, ob1, oW2, ob2, oW3, ob3, np;
  DevBuf P, G, M, V, Pb;  // Pb: bf16 copies of the weights (same offsets)
  DevBuf PbT;             // bf16 weights transposed (out x in per layer, same offsets): the forward pass's B
                          // operand with K contiguous
  DevBuf mu, sg;
  DevBuf lists, llen, cent;
  std::vector<uint32_t> h_entry;
  float margin = 1.5f, fallback_p = 0.f;
  uint32_t Lmin = 16, Lmax = 512, L_plain = 512;
  uint32_t min_llen = 0;  // shortest entry list (0 when a cluster is empty)
  int steps = 0;
  bool ready = false;

  void layout(uint32_t d, uint32_t c) {
    D = d;
    C = c;
    size_t o = 0;
    oW1 = o;
    o += (size_t)D * HID;
    ob1 = o;
    o += HID;
    oW2 = o;
    o += (size_t)HID * HID;
    ob2 = o;
    o += HID;
    oW3 = o;
    o += (size_t)HID * (C + 1);
    ob3 = o;
    o += C + 1;
    np = o;
  }
};

void learn_free(wv_ctx *c) {
  if (!c->learn) return;
  LearnState *L = static_cast<LearnState *>(c->learn);
  for (DevBuf *b : {&L->P, &L->G, &L->M, &L->V, &L->Pb, &L->PbT, &L->mu, &L->sg, &L->lists, &L->llen, &L->cent})
    b->release();
  delete L;
  c->learn = nullptr;
}

namespace {

struct Work {  // activations and gradients of one batch
  __nv_bfloat16 *Xb, *H1b, *H2b, *dOb, *dZ2b, *dZ1b;
  float *H1, *H2, *O, *dO, *dH2, *dZ2, *dH1, *dZ1;
};

// `pfx` names the buffers (a captured plan keeps its own); `grads`: the
// backward-pass buffers too
int alloc_work(wv_ctx *c, uint32_t B, uint32_t D, uint32_t C, Work &w, const std::string &pfx = "ml_",
               bool grads = true) {
  cudaError_t e = cudaSuccess;
  auto nm = [&](const char *s) { return (pfx + s); };
  w = Work{};
  w.Xb = c->buf<__nv_bfloat16>(nm("Xb").c_str(), (size_t)B * D, &e);
  w.H1b = c->buf<__nv_bfloat16>(nm("H1b").c_str(), (size_t)B * HID, &e);
  w.H2b = c->buf<__nv_bfloat16>(nm("H2b").c_str(), (size_t)B * HID, &e);
  w.H1 = c->buf<float>(nm("H1").c_str(), (size_t)B * HID, &e);
  w.H2 = c->buf<float>(nm("H2").c_str(), (size_t)B * HID, &e);
  w.O = c->buf<float>(nm("O").c_str(), (size_t)B * (C + 1), &e);
  if (grads) {
    w.dOb = c->buf<__nv_bfloat16>(nm("dOb").c_str(), (size_t)B * (C + 1), &e);
    w.dZ2b = c->buf<__nv_bfloat16>(nm("dZ2b").c_str(), (size_t)B * HID, &e);
    w.dZ1b = c->buf<__nv_bfloat16>(nm("dZ1b").c_str(), (size_t)B * HID, &e);
    w.dO = c->buf<float>(nm("dO").c_str(), (size_t)B * (C + 1), &e);
    w.dH2 = c->buf<float>(nm("dH2").c_str(), (size_t)B * HID, &e);
    w.dZ2 = c->buf<float>(nm("dZ2").c_str(), (size_t)B * HID, &e);
    w.dH1 = c->buf<float>(nm("dH1").c_str(), (size_t)B * HID, &e);
    w.dZ1 = c->buf<float>(nm("dZ1").c_str(), (size_t)B * HID, &e);
  }
  WV_CUDA(c, e);
  return WV_OK;
}

GemmArgs gm(const __nv_bfloat16 *A, long long sam, long long sak, const __nv_bfloat16 *B, long long sbk, long long sbn,
            float *C, __nv_bfloat16 *Cb, long long ldc, const float *bias, int relu, int M, int N, int K) {
  GemmArgs g;
  g.A = A;
  g.sam = sam;
  g.sak = sak;
  g.B = B;
  g.sbk = sbk;
  g.sbn = sbn;
  g.C = C;
  g.Cb = Cb;
  g.ldc = ldc;
  g.bias = bias;
  g.relu = relu;
  g.M = M;
  g.N = N;
  g.K = K;
  return g;
}

inline unsigned nblk(size_t n, unsigned t = 256) { return (unsigned)((n + t - 1) / t); }

// forward pass of B rows of x (rows: optional gather list); O = outputs
int forward(wv_ctx *c, LearnState &S, const float *x, const uint32_t *rows, uint32_t B, Work &w) {
  const float *P = S.P.as<float>();
  const __nv_bfloat16 *Pt = S.PbT.as<__nv_bfloat16>();  // W^T: B(k, n) = Pt[n * K + k]
  k_gather_norm<<<nblk((size_t)B * S.D), 256, 0, c->stream>>>(x, rows, B, S.D, S.mu.as<float>(), S.sg.as<float>(),
                                                              w.Xb);
  WV_CUDA(c, gemm_bf16_umma(gm(w.Xb, S.D, 1, Pt + S.oW1, 1, S.D, w.H1, w.H1b, HID, P + S.ob1, 1, B, HID, S.D),
                            c->d_status(), c->stream));
  WV_CUDA(c, gemm_bf16_umma(gm(w.H1b, HID, 1, Pt + S.oW2, 1, HID, w.H2, w.H2b, HID, P + S.ob2, 1, B, HID, HID),
                            c->d_status(), c->stream));
  WV_CUDA(c, gemm_bf16_umma(gm(w.H2b, HID, 1, Pt + S.oW3, 1, HID, w.O, nullptr, S.C + 1, P + S.ob3, 0, B, S.C + 1, HID),
                            c->d_status(), c->stream));
  return WV_OK;
}

// loss and gradients (into S.G) of a batch; loss[0] ce, loss[1] mse
int backward(wv_ctx *c, LearnState &S, const uint32_t *yc, const float *yr, const uint32_t *rows, uint32_t B,
             float lam, Work &w, float *loss) {
  const __nv_bfloat16 *Pb = S.Pb.as<__nv_bfloat16>();
  float *G = S.G.as<float>();
  const uint32_t W = S.C + 1;
  k_loss_grad<<<nblk((size_t)B * 32), 256, 0, c->stream>>>(w.O, B, S.C, yc, yr, rows, lam, w.dO, w.dOb, loss);
  // layer 3
  WV_CUDA(c, gemm_bf16_umma(gm(w.H2b, 1, HID, w.dOb, W, 1, G + S.oW3, nullptr, W, nullptr, 0, HID, W, B), c->d_status(), c->stream));
  k_colsum<<<nblk(W), 256, 0, c->stream>>>(w.dO, B, W, G + S.ob3);
  WV_CUDA(c, gemm_bf16_umma(gm(w.dOb, W, 1, Pb + S.oW3, 1, W, w.dH2, nullptr, HID, nullptr, 0, B, HID, W), c->d_status(), c->stream));
  k_relu_bwd<<<nblk((size_t)B * HID), 256, 0, c->stream>>>(w.dH2, w.H2, (size_t)B * HID, w.dZ2, w.dZ2b);
  // layer 2
  WV_CUDA(c, gemm_bf16_umma(gm(w.H1b, 1, HID, w.dZ2b, HID, 1, G + S.oW2, nullptr, HID, nullptr, 0, HID, HID, B), c->d_status(), c->stream));
  k_colsum<<<nblk(HID), 256, 0, c->stream>>>(w.dZ2, B, HID, G + S.ob2);
  WV_CUDA(c, gemm_bf16_umma(gm(w.dZ2b, HID, 1, Pb + S.oW2, 1, HID, w.dH1, nullptr, HID, nullptr, 0, B, HID, HID), c->d_status(), c->stream));
  k_relu_bwd<<<nblk((size_t)B * HID), 256, 0, c->stream>>>(w.dH1, w.H1, (size_t)B * HID, w.dZ1, w.dZ1b);
  // layer 1
  WV_CUDA(c, gemm_bf16_umma(gm(w.Xb, 1, S.D, w.dZ1b, HID, 1, G + S.oW1, nullptr, HID, nullptr, 0, S.D, HID, B), c->d_status(), c->stream));
  k_colsum<<<nblk(HID), 256, 0, c->stream>>>(w.dZ1, B, HID, G + S.ob1);
  WV_CUDA(c, cudaGetLastError());
  return WV_OK;
}

int refresh_bf16(wv_ctx *c, LearnState &S) {
  k_to_bf16<<<nblk(S.np), 256, 0, c->stream>>>(S.P.as<float>(), S.np, S.Pb.as<__nv_bfloat16>());
  WV_CUDA(c, cudaGetLastError());
  const float *P = S.P.as<float>();
  __nv_bfloat16 *T = S.PbT.as<__nv_bfloat16>();
  const size_t offs[3] = {S.oW1, S.oW2, S.oW3};
  const uint32_t rows[3] = {S.D, HID, HID}, cols[3] = {HID, HID, S.C + 1};
  for (int l = 0; l < 3; l++) {
    k_transpose_bf16<<<nblk((size_t)rows[l] * cols[l]), 256, 0, c->stream>>>(P + offs[l], rows[l], cols[l],
                                                                             T + offs[l]);
    WV_CUDA(c, cudaGetLastError());
  }
  return WV_OK;
}

int ensure_params(wv_ctx *c, LearnState &S) {
  WV_CUDA(c, S.P.ensure(S.np * 4));
  WV_CUDA(c, S.G.ensure(S.np * 4));
  WV_CUDA(c, S.M.ensure(S.np * 4));
  WV_CUDA(c, S.V.ensure(S.np * 4));
  WV_CUDA(c, S.Pb.ensure(S.np * 2));
  WV_CUDA(c, S.PbT.ensure(S.np * 2));
  return WV_OK;
}

// He-style initialisation from the context's own generator (host), biases 0
void init_params(LearnState &S, uint32_t seed, std::vector<float> &h) {
  h.assign(S.np, 0.f);
  std::mt19937 rng(seed);
  std::normal_distribution<float> nd(0.f, 1.f);
  auto fill = [&](size_t off, size_t cnt, float sd) {
    for (size_t i = 0; i < cnt; i++) h[off + i] = nd(rng) * sd;
  };
  fill(S.oW1, (size_t)S.D * HID, std::sqrt(2.f / S.D));
  fill(S.oW2, (size_t)HID * HID, std::sqrt(2.f / HID));
  fill(S.oW3, (size_t)HID * (S.C + 1), std::sqrt(1.f / HID));
}

LearnState &state(wv_ctx *c) {
  if (!c->learn) c->learn = new LearnState();
  return *static_cast<LearnState *>(c->learn);
}

// runs the plain (or seeded) batched search on device queries; ids out (device)
int search_dev(wv_ctx *c, const float *dq, uint32_t nq, const uint32_t *dseeds, uint32_t seed_stride,
               const uint32_t *dL, uint32_t L, uint32_t Lmax, uint32_t K, uint32_t *dout, wv_counters *cnt);

}  // namespace

// ================================================================ fit
int learn_fit(wv_ctx *c, const float *train_q, uint32_t nt, const LearnParams &p, LearnReport *rep) {
  WV_CHECK(c, c->n > 0 && c->gn == c->n, WV_ERR_STATE, "learning needs the base and the search graph");
  WV_CHECK(c, p.clusters >= 2 && p.clusters <= 256, WV_ERR_ARG, "clusters must be in [2, 256]");
  WV_CHECK(c, nt >= 64, WV_ERR_ARG, "need at least 64 training queries");
  WV_CHECK(c, (size_t)p.clusters * (c->d + 1) * 4 <= 160 * 1024, WV_ERR_LIMIT, "clusters x d too large");
  LearnState &S = state(c);
  S.ready = false;
  S.layout(c->d, p.clusters);
  // the traces and labels come from the plain search in the exact traversal
  // (the judge), whatever expansion width later searches use
  struct KeepParents {
    wv_ctx *c;
    uint32_t p;
    ~KeepParents() { c->parents = p; }
  } keep_parents{c, c->parents};
  c->parents = 0;
  const uint32_t C = p.clusters, d = c->d, n = c->n;
  cudaError_t e = cudaSuccess;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, c->stream);
  // ---- k-means on the base (centroids start at evenly spaced rows)
  WV_CUDA(c, S.cent.ensure((size_t)C * d * 4));
  std::vector<float> hc((size_t)C * d);
  for (uint32_t k = 0; k < C; k++)
    WV_CUDA(c, cudaMemcpyAsync(S.cent.as<float>() + (size_t)k * d, c->base.as<float>() + (size_t)(k * (n / C)) * d,
                               d * 4, cudaMemcpyDeviceToDevice, c->stream));
  uint32_t *asg = c->buf<uint32_t>("km_asg", n, &e);
  float *adist = c->buf<float>("km_dist", n, &e);
  float *sum = c->buf<float>("km_sum", (size_t)C * d, &e);
  uint32_t *cnt = c->buf<uint32_t>("km_cnt", C, &e);
  WV_CUDA(c, e);
  const size_t csm = (size_t)C * (d + 1) * 4;
  WV_CUDA(c, cudaFuncSetAttribute(k_km_assign, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)csm));
  std::vector<uint32_t> hcnt(C);
  for (uint32_t it = 0; it < p.kmeans_iters; it++) {
    k_km_assign<<<c->sms * 8, 256, csm, c->stream>>>(c->base.as<float>(), n, d, S.cent.as<float>(), C, asg, adist);
    WV_CUDA(c, cudaMemsetAsync(sum, 0, (size_t)C * d * 4, c->stream));
    WV_CUDA(c, cudaMemsetAsync(cnt, 0, (size_t)C * 4, c->stream));
    k_km_accum<<<nblk((size_t)n * d), 256, 0, c->stream>>>(c->base.as<float>(), n, d, asg, sum, cnt);
    WV_CUDA(c, cudaMemcpyAsync(hc.data(), sum, (size_t)C * d * 4, cudaMemcpyDeviceToHost, c->stream));
    WV_CUDA(c, cudaMemcpyAsync(hcnt.data(), cnt, (size_t)C * 4, cudaMemcpyDeviceToHost, c->stream));
    WV_CUDA(c, cudaStreamSynchronize(c->stream));
    std::vector<float> old((size_t)C * d);
    WV_CUDA(c, cudaMemcpy(old.data(), S.cent.p, (size_t)C * d * 4, cudaMemcpyDeviceToHost));
    for (uint32_t k = 0; k < C; k++)
      for (uint32_t j = 0; j < d; j++)
        hc[(size_t)k * d + j] = hcnt[k] ? hc[(size_t)k * d + j] / hcnt[k] : old[(size_t)k * d + j];
    WV_CUDA(c, cudaMemcpyAsync(S.cent.p, hc.data(), (size_t)C * d * 4, cudaMemcpyHostToDevice, c->stream));
  }
  k_km_assign<<<c->sms * 8, 256, csm, c->stream>>>(c->base.as<float>(), n, d, S.cent.as<float>(), C, asg, adist);
  WV_CUDA(c, cudaGetLastError());
  // ---- entry lists: nearest member first, then members in a fixed
  // pseudo-random order (hash of the id)
  std::vector<uint32_t> ha(n);
  std::vector<float> hd(n);
  WV_CUDA(c, cudaMemcpyAsync(ha.data(), asg, (size_t)n * 4, cudaMemcpyDeviceToHost, c->stream));
  WV_CUDA(c, cudaMemcpyAsync(hd.data(), adist, (size_t)n * 4, cudaMemcpyDeviceToHost, c->stream));
  WV_CUDA(c, cudaStreamSynchronize(c->stream));
  S.SL = p.list_len;
  S.h_assign = ha;
  std::vector<std::vector<uint32_t>> mem(C);
  for (uint32_t i = 0; i < n; i++) mem[ha[i]].push_back(i);
  std::vector<uint32_t> hl((size_t)C * S.SL, 0), hll(C, 0);
  S.h_entry.assign(C, 0);
  for (uint32_t k = 0; k < C; k++) {
    auto &m = mem[k];
    if (m.empty()) continue;
    uint32_t best = m[0];
    for (uint32_t i : m)
      if (hd[i] < hd[best] || (hd[i] == hd[best] && i < best)) best = i;
    S.h_entry[k] = best;
    std::vector<std::pair<uint32_t, uint32_t>> ord;
    for (uint32_t i : m)
      if (i != best) ord.push_back({i * 2654435761u, i});
    std::sort(ord.begin(), ord.end());
    uint32_t t = 0;
    hl[(size_t)k * S.SL + t++] = best;
    for (size_t j = 0; j < ord.size() && t < S.SL; j++) hl[(size_t)k * S.SL + t++] = ord[j].second;
    hll[k] = t;
  }
  S.min_llen = *std::min_element(hll.begin(), hll.end());
  WV_CUDA(c, S.lists.ensure(hl.size() * 4));
  WV_CUDA(c, S.llen.ensure((size_t)C * 4));
  WV_CUDA(c, cudaMemcpyAsync(S.lists.p, hl.data(), hl.size() * 4, cudaMemcpyHostToDevice, c->stream));
  WV_CUDA(c, cudaMemcpyAsync(S.llen.p, hll.data(), (size_t)C * 4, cudaMemcpyHostToDevice, c->stream));
  // ---- traces: the plain search answers every training query
  float *dq = c->buf<float>("ml_tq", (size_t)nt * d, &e);
  uint32_t *pseeds = c->buf<uint32_t>("ml_pseeds", (size_t)nt * p.L_trace, &e);
  uint32_t *pans = c->buf<uint32_t>("ml_pans", (size_t)nt * 10, &e);
  WV_CUDA(c, e);
  WV_CUDA(c, cudaMemcpyAsync(dq, train_q, (size_t)nt * d * 4, cudaMemcpyHostToDevice, c->stream));
  int rc = draw_seeds_rand_device(c, nt, nullptr, p.L_trace, p.L_trace, pseeds, p.L_trace);
  if (rc) return rc;
  rc = search_dev(c, dq, nt, pseeds, p.L_trace, nullptr, p.L_trace, p.L_trace, 10, pans, nullptr);
  if (rc) return rc;
  std::vector<uint32_t> hans((size_t)nt * 10);
  WV_CUDA(c, cudaMemcpyAsync(hans.data(), pans, hans.size() * 4, cudaMemcpyDeviceToHost, c->stream));
  WV_CUDA(c, cudaStreamSynchronize(c->stream));
  std::vector<uint32_t> yc(nt);
  for (uint32_t q = 0; q < nt; q++) yc[q] = ha[hans[(size_t)q * 10]];
  // beam labels: smallest L of the grid whose cluster-seeded answer keeps
  // >= 9 of the 10 plain ids
  const std::vector<uint32_t> grid = {16, 24, 32, 48, 64, 96, 128, 192, 256, 384, 512};
  std::vector<float> yr(nt, std::log2((float)grid.back()));
  std::vector<char> done(nt, 0);
  uint32_t *dlab = c->buf<uint32_t>("ml_lab", nt, &e);
  uint32_t *gseeds = c->buf<uint32_t>("ml_gseeds", (size_t)nt * grid.back(), &e);
  uint32_t *gans = c->buf<uint32_t>("ml_gans", (size_t)nt * 10, &e);
  WV_CUDA(c, e);
  WV_CUDA(c, cudaMemcpyAsync(dlab, yc.data(), (size_t)nt * 4, cudaMemcpyHostToDevice, c->stream));
  std::vector<uint32_t> hg((size_t)nt * 10);
  for (uint32_t L : grid) {
    if (L >= n || L > S.SL + p.L_trace) break;
    k_cluster_seeds<<<nblk(nt), 256, 0, c->stream>>>(dlab, nt, S.lists.as<uint32_t>(), S.SL, S.llen.as<uint32_t>(), L,
                                                    pseeds, p.L_trace, gseeds);
    rc = search_dev(c, dq, nt, gseeds, L, nullptr, L, L, 10, gans, nullptr);
    if (rc) return rc;
    WV_CUDA(c, cudaMemcpyAsync(hg.data(), gans, hg.size() * 4, cudaMemcpyDeviceToHost, c->stream));
    WV_CUDA(c, cudaStreamSynchronize(c->stream));
    for (uint32_t q = 0; q < nt; q++) {
      if (done[q]) continue;
      int hit = 0;
      for (int a = 0; a < 10; a++)
        for (int b = 0; b < 10; b++) hit += hg[(size_t)q * 10 + a] == hans[(size_t)q * 10 + b];
      if (hit >= 9) {
        done[q] = 1;
        yr[q] = std::log2((float)L);
      }
    }
  }
  // ---- normalisation and split (last 10% held out for calibration)
  std::vector<float> mu(d, 0.f), sg(d, 0.f);
  for (uint32_t q = 0; q < nt; q++)
    for (uint32_t j = 0; j < d; j++) mu[j] += train_q[(size_t)q * d + j];
  for (uint32_t j = 0; j < d; j++) mu[j] /= nt;
  for (uint32_t q = 0; q < nt; q++)
    for (uint32_t j = 0; j < d; j++) {
      const float t = train_q[(size_t)q * d + j] - mu[j];
      sg[j] += t * t;
    }
  for (uint32_t j = 0; j < d; j++) sg[j] = std::sqrt(sg[j] / nt) + 1e-6f;
  WV_CUDA(c, S.mu.ensure(d * 4));
  WV_CUDA(c, S.sg.ensure(d * 4));
  WV_CUDA(c, cudaMemcpyAsync(S.mu.p, mu.data(), d * 4, cudaMemcpyHostToDevice, c->stream));
  WV_CUDA(c, cudaMemcpyAsync(S.sg.p, sg.data(), d * 4, cudaMemcpyHostToDevice, c->stream));
  const uint32_t nval = std::max<uint32_t>(nt / 10, 1), ntr = nt - nval;
  float *dyr = c->buf<float>("ml_yr", nt, &e);
  uint32_t *drows = c->buf<uint32_t>("ml_rows", nt, &e);
  float *dloss = c->buf<float>("ml_loss", 4, &e);
  WV_CUDA(c, e);
  WV_CUDA(c, cudaMemcpyAsync(dyr, yr.data(), (size_t)nt * 4, cudaMemcpyHostToDevice, c->stream));
  // ---- train
  rc = ensure_params(c, S);
  if (rc) return rc;
  std::vector<float> hp;
  init_params(S, p.seed, hp);
  WV_CUDA(c, cudaMemcpyAsync(S.P.p, hp.data(), S.np * 4, cudaMemcpyHostToDevice, c->stream));
  WV_CUDA(c, cudaMemsetAsync(S.M.p, 0, S.np * 4, c->stream));
  WV_CUDA(c, cudaMemsetAsync(S.V.p, 0, S.np * 4, c->stream));
  Work w;
  rc = alloc_work(c, std::max(p.batch, nval), d, C, w);
  if (rc) return rc;
  std::vector<uint32_t> perm(ntr);
  std::iota(perm.begin(), perm.end(), 0u);
  std::mt19937 rng(p.seed);
  S.steps = 0;
  float last[2] = {0, 0};
  for (uint32_t ep = 0; ep < p.epochs; ep++) {
    std::shuffle(perm.begin(), perm.end(), rng);
    WV_CUDA(c, cudaMemcpyAsync(drows, perm.data(), (size_t)ntr * 4, cudaMemcpyHostToDevice, c->stream));
    for (uint32_t b0 = 0; b0 + p.batch <= ntr; b0 += p.batch) {
      rc = refresh_bf16(c, S);
      if (rc) return rc;
      rc = forward(c, S, dq, drows + b0, p.batch, w);
      if (rc) return rc;
      WV_CUDA(c, cudaMemsetAsync(dloss, 0, 8, c->stream));
      rc = backward(c, S, dlab, dyr, drows + b0, p.batch, p.lam, w, dloss);
      if (rc) return rc;
      S.steps++;
      const float c1 = 1.f - std::pow(0.9f, (float)S.steps), c2 = 1.f - std::pow(0.999f, (float)S.steps);
      k_adam<<<nblk(S.np), 256, 0, c->stream>>>(S.P.as<float>(), S.G.as<float>(), S.M.as<float>(), S.V.as<float>(),
                                               S.np, p.lr, 0.9f, 0.999f, 1e-8f, c1, c2);
      WV_CUDA(c, cudaGetLastError());
    }
    WV_CUDA(c, cudaMemcpyAsync(last, dloss, 8, cudaMemcpyDeviceToHost, c->stream));
    WV_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  rc = refresh_bf16(c, S);
  if (rc) return rc;
  // ---- calibration on the held-out queries: the smallest beam margin whose
  // answers keep the plain answers at the target rate
  S.Lmin = p.L_min;
  S.Lmax = p.L_max;
  S.L_plain = p.L_trace;
  S.fallback_p = p.fallback_p;
  S.ready = true;
  const float margins[] = {1.0f, 1.25f, 1.5f, 2.0f, 2.5f, 3.0f, 4.0f, 6.0f};
  float chosen = margins[7], chosen_rate = 0.f;
  std::vector<uint32_t> vans((size_t)nval * 10);
  for (float mg : margins) {
    S.margin = mg;
    rc = learn_search(c, dq + (size_t)ntr * d, nval, 10, gans, nullptr, nullptr, pseeds + (size_t)ntr * p.L_trace,
                      nullptr);
    if (rc) return rc;
    WV_CUDA(c, cudaMemcpyAsync(vans.data(), gans, vans.size() * 4, cudaMemcpyDeviceToHost, c->stream));
    WV_CUDA(c, cudaStreamSynchronize(c->stream));
    size_t hit = 0;
    for (uint32_t q = 0; q < nval; q++)
      for (int a = 0; a < 10; a++)
        for (int b = 0; b < 10; b++) hit += vans[(size_t)q * 10 + a] == hans[(size_t)(ntr + q) * 10 + b];
    const float rate = (float)hit / (nval * 10.f);
    if (rate >= p.target_agreement) {
      chosen = mg;
      chosen_rate = rate;
      break;
    }
    chosen_rate = rate;
  }
  S.margin = chosen;
  cudaEventRecord(e1, c->stream);
  cudaEventSynchronize(e1);
  if (rep) {
    *rep = LearnReport{};
    rep->loss_ce = last[0];
    rep->loss_mse = last[1];
    rep->steps = S.steps;
    rep->margin = chosen;
    rep->val_agreement = chosen_rate;
    cudaEventElapsedTime(&rep->ms, e0, e1);
    size_t lab_done = 0;
    double lmean = 0;
    for (uint32_t q = 0; q < nt; q++) {
      lab_done += done[q];
      lmean += std::exp2(yr[q]);
    }
    rep->labelled = (uint32_t)lab_done;
    rep->mean_label_L = (float)(lmean / nt);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return WV_OK;
}

// ================================================================ search
namespace {
int search_dev(wv_ctx *c, const float *dq, uint32_t nq, const uint32_t *dseeds, uint32_t seed_stride,
               const uint32_t *dL, uint32_t L, uint32_t Lmax, uint32_t K, uint32_t *dout, wv_counters *cnt) {
  return run_search_device(c, dq, nq, dseeds, seed_stride, dL, nullptr, L, K, Lmax, dout, nullptr, K, cnt);
}
}  // namespace

int learn_search(wv_ctx *c, const float *dq, uint32_t nq, uint32_t K, uint32_t *dout, float *ddist,
                 wv_counters *counters, const uint32_t *d_plain_seeds, uint32_t *d_Lq_out) {
  WV_CHECK(c, c->learn && state(c).ready, WV_ERR_STATE, "no trained model (call wv_learn_fit)");
  LearnState &S = state(c);
  WV_CHECK(c, S.D == c->d, WV_ERR_STATE, "model trained for d=%u", S.D);
  cudaError_t e = cudaSuccess;
  const uint32_t stride = std::max(S.Lmax, S.L_plain);
  uint32_t *seeds = c->buf<uint32_t>("ls_seeds", (size_t)nq * stride, &e);
  uint32_t *Lq = c->buf<uint32_t>("ls_Lq", nq, &e);
  uint32_t *fb = c->buf<uint32_t>("ls_fb", 4, &e);
  WV_CUDA(c, e);
  Work w;
  int rc = alloc_work(c, nq, S.D, S.C, w);
  if (rc) return rc;
  rc = forward(c, S, dq, nullptr, nq, w);
  if (rc) return rc;
  WV_CUDA(c, cudaMemsetAsync(fb, 0, 4, c->stream));
  k_learn_seeds<<<nblk(nq, 128), 128, 0, c->stream>>>(w.O, nq, S.C, S.lists.as<uint32_t>(), S.SL, S.llen.as<uint32_t>(),
                                                 S.margin, S.Lmin, S.Lmax, S.fallback_p, S.L_plain, d_plain_seeds,
                                                 seeds, stride, Lq, K, fb);
  WV_CUDA(c, cudaGetLastError());
  if (d_Lq_out) WV_CUDA(c, cudaMemcpyAsync(d_Lq_out, Lq, (size_t)nq * 4, cudaMemcpyDeviceToDevice, c->stream));
  // without the fallback no query's beam exceeds Lmax: size the kernel for it
  const uint32_t Lcap = (d_plain_seeds && S.fallback_p > 0.f) ? stride : S.Lmax;
  return run_search_device(c, dq, nq, seeds, stride, Lq, nullptr, 0, K, Lcap, dout, ddist, K, counters);
}

int learn_prepare(wv_ctx *c, const char *pfx, uint32_t nq_max, uint32_t *Lcap, uint32_t *stride) {
  WV_CHECK(c, c->learn && state(c).ready, WV_ERR_STATE, "no trained model (call wv_learn_fit)");
  LearnState &S = state(c);
  WV_CHECK(c, S.D == c->d, WV_ERR_STATE, "model trained for d=%u", S.D);
  cudaError_t e = cudaSuccess;
  const std::string p(pfx);
  *stride = std::max(S.Lmax, S.L_plain);
  c->buf<uint32_t>((p + "seeds").c_str(), (size_t)nq_max * *stride, &e);
  c->buf<uint32_t>((p + "Lq").c_str(), nq_max, &e);
  c->buf<uint32_t>((p + "order").c_str(), nq_max, &e);
  c->buf<uint32_t>((p + "fb").c_str(), 4, &e);
  WV_CUDA(c, e);
  Work w;
  int rc = alloc_work(c, nq_max, S.D, S.C, w, p, false);
  if (rc) return rc;
  *Lcap = S.fallback_p > 0.f ? *stride : S.Lmax;
  return WV_OK;
}

int learn_enqueue(wv_ctx *c, const char *pfx, const float *dq, uint32_t nq_max, const uint32_t *d_nq, uint32_t K,
                  const uint32_t *d_K, uint32_t *dout, float *ddist, uint32_t out_stride,
                  const uint32_t *d_plain_seeds, SearchShape shape, int blocks, const SearchScratch &scr,
                  cudaEvent_t ev0, cudaEvent_t ev1) {
  LearnState &S = state(c);
  cudaError_t e = cudaSuccess;
  const std::string p(pfx);
  const uint32_t stride = std::max(S.Lmax, S.L_plain);
  uint32_t *seeds = c->buf<uint32_t>((p + "seeds").c_str(), (size_t)nq_max * stride, &e);
  uint32_t *Lq = c->buf<uint32_t>((p + "Lq").c_str(), nq_max, &e);
  uint32_t *order = c->buf<uint32_t>((p + "order").c_str(), nq_max, &e);
  uint32_t *fb = c->buf<uint32_t>((p + "fb").c_str(), 4, &e);
  WV_CUDA(c, e);
  Work w;
  int rc = alloc_work(c, nq_max, S.D, S.C, w, p, false);
  if (rc) return rc;
  rc = forward(c, S, dq, nullptr, nq_max, w);
  if (rc) return rc;
  WV_CUDA(c, cudaMemsetAsync(fb, 0, 4, c->stream));
  k_learn_seeds<<<nblk(nq_max, 128), 128, 0, c->stream>>>(
      w.O, nq_max, S.C, S.lists.as<uint32_t>(), S.SL, S.llen.as<uint32_t>(), S.margin, S.Lmin, S.Lmax, S.fallback_p,
      S.L_plain, d_plain_seeds, seeds, stride, Lq, K, fb);
  WV_CUDA(c, cudaGetLastError());
  const uint32_t Lcap = S.fallback_p > 0.f ? stride : S.Lmax;
  SearchArgs a = search_args(c, dq, nq_max, d_nq, seeds, stride, Lq, d_K, 0, K, Lcap, dout, ddist, out_stride);
  a.order = order;
  if (scr.visited) {
    a.visited = scr.visited;
    a.touched = scr.touched;
    a.words = scr.words;
  }
  if (ev0) WV_CUDA(c, record_event(ev0, c->stream));
  rc = search_enqueue(c, a, shape, blocks);
  if (rc) return rc;
  if (ev1) WV_CUDA(c, record_event(ev1, c->stream));
  return WV_OK;
}

int learn_grad(wv_ctx *c, const float *x, const uint32_t *yc, const float *yr, uint32_t B, uint32_t C,
               const float *params, float lam, float *grad, float *loss) {
  LearnState &S = state(c);
  S.layout(c->d ? c->d : 0, C);
  int rc = ensure_params(c, S);
  if (rc) return rc;
  cudaError_t e = cudaSuccess;
  float *dx = c->buf<float>("lg_x", (size_t)B * S.D, &e);
  uint32_t *dyc = c->buf<uint32_t>("lg_yc", B, &e);
  float *dyr = c->buf<float>("lg_yr", B, &e);
  float *dl = c->buf<float>("lg_loss", 4, &e);
  WV_CUDA(c, e);
  std::vector<float> ones(S.D, 1.f), zeros(S.D, 0.f);
  WV_CUDA(c, S.mu.ensure(S.D * 4));
  WV_CUDA(c, S.sg.ensure(S.D * 4));
  WV_CUDA(c, cudaMemcpyAsync(S.mu.p, zeros.data(), S.D * 4, cudaMemcpyHostToDevice, c->stream));
  WV_CUDA(c, cudaMemcpyAsync(S.sg.p, ones.data(), S.D * 4, cudaMemcpyHostToDevice, c->stream));
  WV_CUDA(c, cudaMemcpyAsync(dx, x, (size_t)B * S.D * 4, cudaMemcpyHostToDevice, c->stream));
  WV_CUDA(c, cudaMemcpyAsync(dyc, yc, (size_t)B * 4, cudaMemcpyHostToDevice, c->stream));
  WV_CUDA(c, cudaMemcpyAsync(dyr, yr, (size_t)B * 4, cudaMemcpyHostToDevice, c->stream));
  WV_CUDA(c, cudaMemcpyAsync(S.P.p, params, S.np * 4, cudaMemcpyHostToDevice, c->stream));
  rc = refresh_bf16(c, S);
  if (rc) return rc;
  Work w;
  rc = alloc_work(c, B, S.D, C, w);
  if (rc) return rc;
  rc = forward(c, S, dx, nullptr, B, w);
  if (rc) return rc;
  WV_CUDA(c, cudaMemsetAsync(dl, 0, 8, c->stream));
  rc = backward(c, S, dyc, dyr, nullptr, B, lam, w, dl);
  if (rc) return rc;
  WV_CUDA(c, cudaMemcpyAsync(grad, S.G.p, S.np * 4, cudaMemcpyDeviceToHost, c->stream));
  WV_CUDA(c, cudaMemcpyAsync(loss, dl, 8, cudaMemcpyDeviceToHost, c->stream));
  WV_CUDA(c, cudaStreamSynchronize(c->stream));
  S.ready = false;
  return WV_OK;
}

int learn_predict(wv_ctx *c, const float *q, uint32_t nq, uint32_t *cluster, float *prob, float *log2L) {
  WV_CHECK(c, c->learn && state(c).ready, WV_ERR_STATE, "no trained model");
  LearnState &S = state(c);
  cudaError_t e = cudaSuccess;
  float *dq = c->buf<float>("lp_q", (size_t)nq * S.D, &e);
  WV_CUDA(c, e);
  WV_CUDA(c, cudaMemcpyAsync(dq, q, (size_t)nq * S.D * 4, cudaMemcpyHostToDevice, c->stream));
  Work w;
  int rc = alloc_work(c, nq, S.D, S.C, w);
  if (rc) return rc;
  rc = forward(c, S, dq, nullptr, nq, w);
  if (rc) return rc;
  std::vector<float> O((size_t)nq * (S.C + 1));
  WV_CUDA(c, cudaMemcpyAsync(O.data(), w.O, O.size() * 4, cudaMemcpyDeviceToHost, c->stream));
  WV_CUDA(c, cudaStreamSynchronize(c->stream));
  for (uint32_t i = 0; i < nq; i++) {
    const float *o = O.data() + (size_t)i * (S.C + 1);
    uint32_t b = 0;
    for (uint32_t k = 1; k < S.C; k++)
      if (o[k] > o[b]) b = k;
    double se = 0;
    for (uint32_t k = 0; k < S.C; k++) se += std::exp((double)o[k] - o[b]);
    if (cluster) cluster[i] = b;
    if (prob) prob[i] = (float)(1.0 / se);
    if (log2L) log2L[i] = o[S.C];
  }
  return WV_OK;
}

int learn_assign(wv_ctx *c, const uint32_t *ids, uint32_t n, uint32_t *cluster) {
  WV_CHECK(c, c->learn && !state(c).h_assign.empty(), WV_ERR_STATE, "no clusters");
  LearnState &S = state(c);
  for (uint32_t i = 0; i < n; i++) {
    WV_CHECK(c, ids[i] < S.h_assign.size(), WV_ERR_ARG, "id %u out of range", ids[i]);
    cluster[i] = S.h_assign[ids[i]];
  }
  return WV_OK;
}

int learn_set_margin(wv_ctx *c, float margin) {
  static_cast<LearnState *>(c->learn)->margin = margin;
  return WV_OK;
}

int learn_set_fallback(wv_ctx *c, float p, uint32_t L_plain) {
  LearnState &S = *static_cast<LearnState *>(c->learn);
  S.fallback_p = p;
  S.L_plain = L_plain;
  return WV_OK;
}

uint32_t learn_plain_beam(wv_ctx *c) {
  if (!c->learn) return 0u;
  const LearnState &S = *static_cast<LearnState *>(c->learn);
  // without the fallback, and with every entry list at least as long as the
  // largest beam, k_learn_seeds never reads a plain seed
  if (!(S.fallback_p > 0.f) && S.min_llen >= S.Lmax) return 0u;
  return S.L_plain;
}

size_t learn_param_count(uint32_t d, uint32_t C) {
  LearnState S;
  S.layout(d, C);
  return S.np;
}

}  // namespace wv
