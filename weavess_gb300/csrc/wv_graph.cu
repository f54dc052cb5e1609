// Graph files and index statistics.
//
// Files: the per-node form of IndexBuilder::save_graph / load_graph
// (src/builder.cpp:918-1089, the branch every KNN-graph index falls through
// to, and INDEX_EXACT_KNNG): an optional entry point (one u32, NSG and
// Vamana), then for every node its degree GK (u32) and GK ids (u32), native
// byte order.  Byte-compatible with the reference in both directions.
//
// Statistics: IndexBuilder::print_index_info (builder.cpp:501-600, 714-780)
//  * degree: max / min / mean out-degree;
//  * conn: the number of depth-first traversals needed to reach every node,
//    starting at the entry point (or node 0) and restarting at the smallest
//    unreached id.  A traversal's reach does not depend on its order, so the
//    GPU runs it as a level-synchronous BFS (frontier kernels) and counts the
//    same restarts;
//  * quality: the mean, over nodes, of the share of the node's first 10 exact
//    neighbours (itself skipped) found in its row, the share taken over
//    min(10, degree, exact-list length) as the reference divides.
#include <algorithm>
#include <cstdio>
#include <utility>
#include <vector>

#include "wv_bfs.cuh"
#include "wv_common.cuh"
#include "wv_ctx.h"

using namespace wv;

namespace {

// one BFS level over the HNSW graph: a node's friends on every layer (layer 0
// rows of width w0; layers 1.. as (count, ids) records of wu + 1 words from
// up_off), as IndexBuilder::DFS walks INDEX_HNSW (builder.cpp:603-625)
__global__ void k_bfs_hnsw(const uint32_t *l0, const uint32_t *deg0, uint32_t w0, const uint32_t *up_off,
                           const uint32_t *up, uint32_t wu, const uint32_t *layers, uint32_t n, const uint32_t *front,
                           uint32_t nfront, uint32_t *bits, uint32_t *next, uint32_t *nnext, int *status) {
  const int lane = threadIdx.x & 31;
  const uint32_t wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t f = wid; f < nfront; f += nw) {
    const uint32_t u = front[f];
    const uint32_t t = layers[u] ? layers[u] : 1u;
    for (uint32_t l = 0; l < t; l++) {
      const uint32_t *row;
      uint32_t dg;
      if (l == 0) {
        row = l0 + (size_t)u * w0;
        dg = min(deg0[u], w0);
      } else {
        const uint32_t *rec = up + (size_t)up_off[u] + (size_t)(l - 1) * (wu + 1);
        dg = min(rec[0], wu);
        row = rec + 1;
      }
      for (uint32_t j = lane; j < dg; j += 32) {
        const uint32_t v = row[j];
        if (v >= n) {
          set_err(status, DEV_BAD_ID);
          continue;
        }
        const uint32_t bit = 1u << (v & 31);
        if (!(atomicOr(bits + (v >> 5), bit) & bit)) next[atomicAdd(nnext, 1u)] = v;
      }
    }
  }
}

// per node: share of its first 10 exact neighbours (itself skipped) in its row
__global__ void k_quality(const uint32_t *ids, const uint32_t *deg, uint32_t w, const uint32_t *ex,
                          const uint32_t *exdeg, uint32_t ew, uint32_t n, float *q) {
  const int lane = threadIdx.x & 31;
  const uint32_t wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t i = wid; i < n; i += nw) {
    const uint32_t *v = ex + (size_t)i * ew;
    uint32_t vl = min(exdeg[i], ew);
    uint32_t v0 = 0;
    if (vl > 0 && v[0] == i) {
      v0 = 1;
      vl--;
    }
    const uint32_t dg = min(deg[i], w);
    uint32_t hits = 0;
    for (uint32_t j = 0; j < 10 && j < vl; j++) {
      const uint32_t target = v[v0 + j];
      bool found = false;
      for (uint32_t k = lane; k < dg && !found; k += 32) found = ids[(size_t)i * w + k] == target;
      hits += __any_sync(FULL, found) ? 1u : 0u;
    }
    if (lane == 0) {
      const uint32_t den = min(min(10u, dg), vl);
      q[i] = den ? (float)hits / (float)den : __int_as_float(0x7fc00000);  // 0/0 as the reference's float division
    }
  }
}

}  // namespace

extern "C" {

int wv_save_graph(wv_ctx *c, const char *path, int with_ep) {
  if (!c || !path) return WV_ERR_ARG;
  WV_CHECK(c, with_ep >= WV_GRAPH_PLAIN && with_ep <= WV_GRAPH_EPS, WV_ERR_ARG,
           "header form %d cannot be saved (HNSW graphs are load-only here)", with_ep);
  WV_CHECK(c, c->fg_n > 0, WV_ERR_STATE, "no built graph");
  const size_t n = c->fg_n, w = c->fg_w;
  std::vector<uint32_t> ids(n * w), deg(n);
  WV_CUDA(c, cudaSetDevice(c->device));
  WV_CUDA(c, cudaMemcpyAsync(ids.data(), c->fg_ids.p, n * w * 4, cudaMemcpyDeviceToHost, c->stream));
  WV_CUDA(c, cudaMemcpyAsync(deg.data(), c->fg_deg.p, n * 4, cudaMemcpyDeviceToHost, c->stream));
  WV_CUDA(c, cudaStreamSynchronize(c->stream));
  FILE *f = fopen(path, "wb");
  WV_CHECK(c, f, WV_ERR_ARG, "cannot open %s for writing", path);
  bool ok = true;
  if (with_ep == WV_GRAPH_EPS) {  // INDEX_SSG: root count, then the roots
    const uint32_t ne = (uint32_t)c->fg_eps.size();
    ok = fwrite(&ne, 4, 1, f) == 1 && fwrite(c->fg_eps.data(), 4, ne, f) == ne;
  } else if (with_ep) {
    ok = fwrite(&c->fg_ep, 4, 1, f) == 1;
  }
  for (size_t i = 0; i < n && ok; i++) {
    const uint32_t gk = deg[i] <= w ? deg[i] : (uint32_t)w;
    ok = fwrite(&gk, 4, 1, f) == 1 && fwrite(ids.data() + i * w, 4, gk, f) == gk;
  }
  ok = (fclose(f) == 0) && ok;
  WV_CHECK(c, ok, WV_ERR_ARG, "writing %s failed", path);
  return WV_OK;
}

int wv_load_graph(wv_ctx *c, const char *path, int with_ep) {
  if (!c || !path) return WV_ERR_ARG;
  WV_CHECK(c, c->n > 0, WV_ERR_STATE, "upload the base first (the graph's node count must match it)");
  FILE *f = fopen(path, "rb");
  WV_CHECK(c, f, WV_ERR_ARG, "cannot open %s", path);
  if (with_ep == WV_GRAPH_HNSW || with_ep == WV_GRAPH_NSW) {  // the whole file, as words
    std::vector<uint32_t> w;
    uint32_t buf[4096];
    size_t got;
    while ((got = fread(buf, 4, 4096, f)) > 0) w.insert(w.end(), buf, buf + got);
    fclose(f);
    if (with_ep == WV_GRAPH_HNSW) return wv_load_hnsw(c, w.data(), w.size());
    // INDEX_NSW (builder.cpp:987-999, 1171-1189): records of (node id, count,
    // ids) until the end; a node's friends are appended in file order.  It
    // becomes a one-layer HNSW graph whose enterpoint is node 0, the node
    // ROUTER_NSW starts from
    const uint32_t n = c->n;
    std::vector<std::vector<uint32_t>> fr(n);
    size_t p = 0;
    while (p + 2 <= w.size()) {
      const uint32_t id = w[p], gk = w[p + 1];
      p += 2;
      WV_CHECK(c, id < n && p + gk <= w.size(), WV_ERR_ARG, "%s: bad NSW record at word %zu", path, p - 2);
      for (uint32_t k = 0; k < gk; k++) WV_CHECK(c, w[p + k] < n, WV_ERR_ARG, "%s: id %u >= n", path, w[p + k]);
      fr[id].insert(fr[id].end(), w.begin() + p, w.begin() + p + gk);
      p += gk;
    }
    std::vector<uint32_t> hw{0u, 0u};
    for (uint32_t v = 0; v < n; v++) {
      hw.push_back(v);
      hw.push_back(1u);
      hw.push_back((uint32_t)fr[v].size());
      hw.insert(hw.end(), fr[v].begin(), fr[v].end());
    }
    return wv_load_hnsw(c, hw.data(), hw.size());
  }
  uint32_t ep = 0;
  std::vector<uint32_t> eps;
  if (with_ep == WV_GRAPH_EPS) {
    uint32_t ne = 0;
    bool ok = fread(&ne, 4, 1, f) == 1 && ne <= c->n;
    if (ok) {
      eps.resize(ne);
      ok = fread(eps.data(), 4, ne, f) == ne;
    }
    for (uint32_t x : eps) ok = ok && x < c->n;
    if (!ok) {
      fclose(f);
      return fail(c, WV_ERR_ARG, "%s: bad root list", path);
    }
  } else if (with_ep && fread(&ep, 4, 1, f) != 1) {
    fclose(f);
    return fail(c, WV_ERR_ARG, "%s: no entry point", path);
  }
  std::vector<std::vector<uint32_t>> rows;
  uint32_t w = 0;
  for (;;) {
    uint32_t gk;
    if (fread(&gk, 4, 1, f) != 1) break;  // end of file, as the reference's loop
    std::vector<uint32_t> r(gk);
    if (gk && fread(r.data(), 4, gk, f) != gk) {
      fclose(f);
      return fail(c, WV_ERR_ARG, "%s: truncated row %zu", path, rows.size());
    }
    w = gk > w ? gk : w;
    rows.push_back(std::move(r));
  }
  fclose(f);
  WV_CHECK(c, rows.size() == c->n, WV_ERR_ARG, "%s holds %zu rows, the base %u", path, rows.size(), c->n);
  w = w ? w : 1;
  std::vector<uint32_t> ids((size_t)c->n * w, 0u), deg(c->n);
  for (size_t i = 0; i < rows.size(); i++) {
    deg[i] = (uint32_t)rows[i].size();
    for (size_t j = 0; j < rows[i].size(); j++) ids[i * w + j] = rows[i][j];
  }
  int rc = wv_upload_graph(c, ids.data(), deg.data(), c->n, w, with_ep == 1 ? ep : 0);
  if (rc == WV_OK) c->eps = eps;
  return rc;
}

int wv_index_info(wv_ctx *c, int use_ep, const uint32_t *exact_ids, const uint32_t *exact_deg, uint32_t exact_width,
                  wv_index_stats *out) {
  if (!c || !out) return WV_ERR_ARG;
  // the HNSW graph: layer-0 degrees and quality, reach over every layer
  // (degree_info / conn_info / graph_quality, builder.cpp:519-527, 573-579, 719-736)
  const bool hnsw = use_ep == WV_GRAPH_HNSW;
  if (hnsw) WV_CHECK(c, c->hnsw.n == c->n && c->n > 0, WV_ERR_STATE, "no HNSW graph");
  else WV_CHECK(c, c->gn == c->n && c->n > 0, WV_ERR_STATE, "no search graph");
  WV_CUDA(c, cudaSetDevice(c->device));
  const uint32_t n = c->n, w = hnsw ? c->hnsw.w0 : c->gw;
  const uint32_t *gids = hnsw ? c->work["hn_l0"].as<uint32_t>() : c->gids.as<uint32_t>();
  const uint32_t *gdeg = hnsw ? c->work["hn_deg0"].as<uint32_t>() : c->gdeg.as<uint32_t>();
  std::vector<uint32_t> deg(n);
  WV_CUDA(c, cudaMemcpyAsync(deg.data(), gdeg, (size_t)n * 4, cudaMemcpyDeviceToHost, c->stream));
  WV_CUDA(c, cudaStreamSynchronize(c->stream));
  wv_index_stats r{};
  r.min_out = 1000000u;
  double sum = 0.0;
  for (uint32_t i = 0; i < n; i++) {
    r.max_out = deg[i] > r.max_out ? deg[i] : r.max_out;
    r.min_out = deg[i] < r.min_out ? deg[i] : r.min_out;
    sum += deg[i];
  }
  r.avg_out = sum / n;
  // connectivity: BFS reach from the root, restarts at the smallest unreached id
  cudaError_t e = cudaSuccess;
  uint32_t *bits = c->buf<uint32_t>("gi_bits", (n + 31) / 32, &e);
  uint32_t *fa = c->buf<uint32_t>("gi_fa", n, &e);
  uint32_t *fb = c->buf<uint32_t>("gi_fb", n, &e);
  uint32_t *cnt = c->buf<uint32_t>("gi_cnt", 4, &e);
  WV_CUDA(c, e);
  WV_CUDA(c, cudaMemsetAsync(bits, 0, (size_t)(n + 31) / 32 * 4, c->stream));
  // the first pass walks from every root (the SSG roots, or the entry point,
  // or node 0), later passes from the smallest unreached id (conn_info,
  // builder.cpp:569-595)
  std::vector<uint32_t> roots;
  if (use_ep == WV_GRAPH_EPS) roots = c->eps;
  else if (hnsw) roots.push_back(c->hnsw.ep);
  else roots.push_back(use_ep ? c->ep : 0u);
  WV_CHECK(c, !roots.empty(), WV_ERR_STATE, "the search graph has no root list");
  for (uint32_t x : roots) WV_CHECK(c, x < n, WV_ERR_ARG, "root %u >= n", x);
  uint32_t conn = 0;
  for (;;) {
    conn++;
    // mark the roots (once each) and make them the frontier
    std::vector<uint32_t> hbits((n + 31) / 32), front;
    WV_CUDA(c, cudaMemcpyAsync(hbits.data(), bits, hbits.size() * 4, cudaMemcpyDeviceToHost, c->stream));
    WV_CUDA(c, cudaStreamSynchronize(c->stream));
    for (uint32_t x : roots) {
      const uint32_t bit = 1u << (x & 31);
      if (!(hbits[x >> 5] & bit)) {
        hbits[x >> 5] |= bit;
        front.push_back(x);
      }
    }
    WV_CUDA(c, cudaMemcpyAsync(bits, hbits.data(), hbits.size() * 4, cudaMemcpyHostToDevice, c->stream));
    WV_CUDA(c, cudaMemcpyAsync(fa, front.data(), front.size() * 4, cudaMemcpyHostToDevice, c->stream));
    WV_CUDA(c, cudaStreamSynchronize(c->stream));
    uint32_t nf = (uint32_t)front.size();
    while (nf) {
      WV_CUDA(c, cudaMemsetAsync(cnt, 0, 4, c->stream));
      const uint32_t blocks = std::min<uint32_t>((nf + 7) / 8, (uint32_t)c->sms * 32);
      if (hnsw)
        k_bfs_hnsw<<<blocks, 256, 0, c->stream>>>(gids, gdeg, w, c->work["hn_upoff"].as<uint32_t>(),
                                                  c->work["hn_up"].as<uint32_t>(), c->hnsw.wu,
                                                  c->work["hn_layers"].as<uint32_t>(), n, fa, nf, bits, fb, cnt,
                                                  c->d_status());
      else
        k_bfs_level<<<blocks, 256, 0, c->stream>>>(gids, gdeg, w, n, fa, nf, bits, fb, cnt, c->d_status());
      WV_CUDA(c, cudaGetLastError());
      WV_CUDA(c, cudaMemcpyAsync(&nf, cnt, 4, cudaMemcpyDeviceToHost, c->stream));
      WV_CUDA(c, cudaStreamSynchronize(c->stream));
      std::swap(fa, fb);
    }
    k_first_unreached<<<1, 1024, 0, c->stream>>>(bits, n, cnt);
    WV_CUDA(c, cudaGetLastError());
    uint32_t root = n;
    WV_CUDA(c, cudaMemcpyAsync(&root, cnt, 4, cudaMemcpyDeviceToHost, c->stream));
    WV_CUDA(c, cudaStreamSynchronize(c->stream));
    if (root >= n) break;
    roots.assign(1, root);
  }
  r.conn = conn;
  r.quality = -1.0;
  if (exact_ids && exact_deg && exact_width) {
    uint32_t *dex = c->buf<uint32_t>("gi_ex", (size_t)n * exact_width, &e);
    uint32_t *dexd = c->buf<uint32_t>("gi_exd", n, &e);
    float *q = c->buf<float>("gi_q", n, &e);
    WV_CUDA(c, e);
    WV_CUDA(c, cudaMemcpyAsync(dex, exact_ids, (size_t)n * exact_width * 4, cudaMemcpyHostToDevice, c->stream));
    WV_CUDA(c, cudaMemcpyAsync(dexd, exact_deg, (size_t)n * 4, cudaMemcpyHostToDevice, c->stream));
    k_quality<<<c->sms * 8, 256, 0, c->stream>>>(gids, gdeg, w, dex, dexd, exact_width, n, q);
    WV_CUDA(c, cudaGetLastError());
    std::vector<float> hq(n);
    WV_CUDA(c, cudaMemcpyAsync(hq.data(), q, (size_t)n * 4, cudaMemcpyDeviceToHost, c->stream));
    WV_CUDA(c, cudaStreamSynchronize(c->stream));
    float s = 0.f;  // mean_quality: a float sum in node order, then / node count (builder.cpp:716-775)
    for (float x : hq) s += x;
    r.quality = s / (float)n;
  }
  *out = r;
  return check_device_status(c, "index info");
}

}  // extern "C"
