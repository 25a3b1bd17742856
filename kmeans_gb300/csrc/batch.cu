// Batched Lloyd (kmgb_lloyd_batched_f32): many independent problems per call.
//
// The reference runs one problem per computeKmeansF call (main/cpp/kmeans.cpp:1316-1361), each
// with its own allocations, shuffle, initialisation and loop; thousands of small problems are
// then bound by launches and allocations. Here problems of the same dimension form one group
// that shares device buffers:
//   * X: every problem's rows start on a 128-row boundary of one matrix (zero rows in between),
//     so each 128-row assignment tile belongs to exactly one problem;
//   * centers: one matrix, problem p owning rows c_off[p] .. c_off[p] + k[p] - 1;
//   * labels: global center indices.
// An iteration is then a fixed number of launches for the whole group: center preparation,
// the grouped FP32 assignment (each tile against its own problem's centers, certified
// margins), the grouped exact re-rank of uncertified rows, the counting sort with tiles that
// never cross a problem (the single-problem stable order, problem after problem), the
// canonical piece sums and the finalize step over all centers, and one warp per problem for
// its SSE and stop rule. A problem whose loop stopped is skipped by the assignment; its update
// recomputes the same centers from the same labels. Results per problem are those of the
// single-problem FP32 tier (and of the oracle) bit for bit: labels, centers, iteration count;
// SSE to FP64 rounding.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <map>
#include <string>
#include <thread>
#include <vector>

#include "../../include/kmeans_gb300.h"
#include "common.cuh"
#include "kernels.h"
#include "tuned_batched.h"

using namespace kmgb;

namespace {

// Predicted GPU time per Lloyd iteration of a problem's rows with one assignment family (0 FP32,
// 1 split BF16): rows x the tuned cost per row of the smallest tuned dimension >= d and the
// smallest tuned k bound >= k (the last ones beyond).
double tuned_cost(int family, int d, int k, long long n) {
  int di = 0, ki = 0;
  const int nd = (int)(sizeof(kTunedDims) / sizeof(kTunedDims[0]));
  const int nk = (int)(sizeof(kTunedKMax) / sizeof(kTunedKMax[0]));
  while (di + 1 < nd && kTunedDims[di] < d) ++di;
  while (ki + 1 < nk && kTunedKMax[ki] < k) ++ki;
  return (double)n * kTunedNsPerRow[family][di][ki];
}

// Tier of every problem: the caller's, or with KMGB_ASSIGN_AUTO one tier per dimension -- the
// family with the smaller predicted time summed over the dimension's problems (the split tier
// only where the tensor-core kernel supports the dimension).
std::vector<int> tiers_of(const kmgb_options& o, const kmgb_problem* problems, int count) {
  std::vector<int> t(count, o.assign_tier);
  if (o.assign_tier != KMGB_ASSIGN_AUTO) return t;
  std::map<int, std::pair<double, double>> cost;  // dimension -> (FP32, split BF16)
  for (int i = 0; i < count; ++i) {
    auto& c = cost[problems[i].d];
    c.first += tuned_cost(0, problems[i].d, problems[i].k, problems[i].n);
    c.second += tuned_cost(1, problems[i].d, problems[i].k, problems[i].n);
  }
  for (int i = 0; i < count; ++i) {
    const auto& c = cost[problems[i].d];
    t[i] = bf16_tc_supported(problems[i].d, 2) && c.second < c.first ? KMGB_ASSIGN_BF16X3
                                                                       : KMGB_ASSIGN_FP32;
  }
  return t;
}

constexpr int kTileRows = 128;       // assignment tile (rows of one problem)
constexpr int kSortTile = 2048;      // counting-sort tile (rows of one problem)
constexpr long long kMaxRows = 1LL << 30;
constexpr long long kMaxHist = 60LL << 20;  // scan capacity of the counting sort
constexpr long long kMaxXBytes = 32LL << 30;

long long rup(long long v, long long m) { return (v + m - 1) / m * m; }

bool on_device(const void* p) {
  if (!p) return false;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

struct DevPool {
  std::vector<void*> ptrs;
  ~DevPool() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <typename T>
  cudaError_t alloc(T** p, size_t count) {
    *p = nullptr;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), sizeof(T) * (count ? count : 1));
    if (e == cudaSuccess) ptrs.push_back(*p);
    return e;
  }
  template <typename T>
  cudaError_t upload(T** p, const std::vector<T>& v, cudaStream_t s) {
    cudaError_t e = alloc(p, v.size());
    if (e != cudaSuccess || v.empty()) return e;
    return cudaMemcpyAsync(*p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, s);
  }
};

struct Fail {
  int code = 0;
  std::string msg;
  bool set(cudaError_t e, int c, const char* where) {
    if (e == cudaSuccess) return false;
    if (!code) {
      code = c;
      msg = std::string("kmgb_lloyd_batched_f32: ") + where + ": " + cudaGetErrorString(e);
    }
    return true;
  }
};

// Initial centers (k x d each, packed) of the group's problems: the given ones, or the
// reference initialisation (shuffle + srand(42) picks), computed on all host cores.
bool initial_centers(const kmgb_problem* pr, const std::vector<int>& ids, int d,
                     std::vector<float>& C0, const std::vector<int>& c_off, Fail& f) {
  const int P = (int)ids.size();
  std::vector<int> bad(P, 0);
  int dev = 0;
  cudaGetDevice(&dev);
  auto work = [&](int lo, int hi) {
    cudaSetDevice(dev);  // worker threads use the caller's device
    std::vector<int> perm, picks;
    for (int i = lo; i < hi; ++i) {
      const kmgb_problem& q = pr[ids[i]];
      float* dst = C0.data() + (size_t)c_off[i] * d;
      if (q.init) {
        if (on_device(q.init)) {
          if (cudaMemcpy(dst, q.init, sizeof(float) * (size_t)q.k * d, cudaMemcpyDeviceToHost) !=
              cudaSuccess)
            bad[i] = 2;
        } else {
          std::memcpy(dst, q.init, sizeof(float) * (size_t)q.k * d);
        }
        continue;
      }
      if (!reference_picks((int)q.n, q.k, picks)) {
        bad[i] = 1;
        continue;
      }
      reference_perm((int)q.n, perm);
      const bool x_dev = on_device(q.X);
      for (int j = 0; j < q.k; ++j) {
        const float* src = q.X + (size_t)perm[picks[j]] * d;
        if (x_dev) {
          if (cudaMemcpy(dst + (size_t)j * d, src, sizeof(float) * d, cudaMemcpyDeviceToHost) !=
              cudaSuccess)
            bad[i] = 2;
        } else {
          std::memcpy(dst + (size_t)j * d, src, sizeof(float) * d);
        }
      }
    }
  };
  int nth = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  nth = std::min(nth, P);
  std::vector<std::thread> th;
  for (int t = 0; t < nth; ++t)
    th.emplace_back(work, (int)((long long)P * t / nth), (int)((long long)P * (t + 1) / nth));
  for (auto& t : th) t.join();
  for (int i = 0; i < P; ++i) {
    if (bad[i] == 1) {
      f.code = KMEANS_ERROR_INITIALIZE;
      f.msg = "kmgb_lloyd_batched_f32: the reference initialisation needs 0 < k <= n";
      return false;
    }
    if (bad[i] == 2) {
      f.code = KMEANS_ERROR_INITIALIZE;
      f.msg = "kmgb_lloyd_batched_f32: copying initial centers failed";
      return false;
    }
  }
  return true;
}

// Host problems' rows into X (rows x ldx): chunks of rows are packed into two alternating
// pinned buffers by host threads (zeros for padding rows and columns) and copied with
// cudaMemcpyAsync while the next chunk is packed.
bool upload_host_rows(const kmgb_problem* pr, const std::vector<int>& ids, int d, long long ldx,
                      long long rows, long long row_pad, const std::vector<long long>& rbeg,
                      const std::vector<long long>& rend, const std::vector<char>& is_dev,
                      float* X, cudaStream_t s, Fail& f) {
  const int E = KMEANS_ERROR_BUILDDATA;
  const long long chunk_rows = std::max<long long>(1, (256LL << 20) / (ldx * 4));
  float* buf[2] = {nullptr, nullptr};
  cudaEvent_t freed[2] = {nullptr, nullptr};
  bool ok = true;
  for (int b = 0; b < 2 && ok; ++b) {
    ok = !f.set(cudaHostAlloc(reinterpret_cast<void**>(&buf[b]),
                              sizeof(float) * chunk_rows * ldx, cudaHostAllocDefault),
                E, "pinned staging") &&
         !f.set(cudaEventCreateWithFlags(&freed[b], cudaEventDisableTiming), E, "staging event");
  }
  const int P = (int)ids.size();
  // problem i's padded region is rows [rbeg[i], pend(i)); the regions tile [0, rows)
  auto pend = [&](int i) { return rbeg[i] + rup(rend[i] - rbeg[i], row_pad); };
  const int nth = (int)std::max(1u, std::min(8u, std::thread::hardware_concurrency()));
  int first = 0;  // first problem whose region ends after the chunk's first row
  for (long long r0 = 0, c = 0; ok && r0 < rows; r0 += chunk_rows, ++c) {
    const long long r1 = std::min(rows, r0 + chunk_rows);
    const int b = (int)(c & 1);
    if (c >= 2 && f.set(cudaEventSynchronize(freed[b]), E, "staging")) {
      ok = false;
      break;
    }
    while (first < P && pend(first) <= r0) ++first;
    float* out = buf[b];
    auto fill = [&](long long a0, long long a1) {  // rows [a0, a1) of X
      int i = first;
      for (long long r = a0; r < a1;) {
        while (pend(i) <= r) ++i;  // r < rows, so some region holds it
        float* dst = out + (size_t)(r - r0) * ldx;
        if (r < rend[i] && !is_dev[i]) {
          const long long stop = std::min(a1, rend[i]);
          const float* src = pr[ids[i]].X + (size_t)(r - rbeg[i]) * d;
          if (ldx == d) {
            std::memcpy(dst, src, sizeof(float) * (size_t)(stop - r) * d);
          } else {
            for (long long t = 0; t < stop - r; ++t) {
              std::memcpy(dst + (size_t)t * ldx, src + (size_t)t * d, sizeof(float) * d);
              std::memset(dst + (size_t)t * ldx + d, 0, sizeof(float) * (ldx - d));
            }
          }
          r = stop;
        } else {  // padding rows (and device problems, copied afterwards) up to the region's end
          const long long stop = std::min(a1, pend(i));
          std::memset(dst, 0, sizeof(float) * (size_t)(stop - r) * ldx);
          r = stop;
        }
      }
    };
    std::vector<std::thread> th;
    const long long n = r1 - r0;
    for (int t = 0; t < nth; ++t) {
      const long long a0 = r0 + n * t / nth, a1 = r0 + n * (t + 1) / nth;
      if (a1 > a0) th.emplace_back(fill, a0, a1);
    }
    for (auto& t : th) t.join();
    ok = !f.set(cudaMemcpyAsync(X + (size_t)r0 * ldx, out, sizeof(float) * (size_t)n * ldx,
                                cudaMemcpyHostToDevice, s),
                E, "data upload") &&
         !f.set(cudaEventRecord(freed[b], s), E, "staging event");
  }
  if (ok) ok = !f.set(cudaStreamSynchronize(s), E, "data upload");
  for (int b = 0; b < 2; ++b) {
    if (freed[b]) cudaEventDestroy(freed[b]);
    if (buf[b]) cudaFreeHost(buf[b]);
  }
  return ok;
}

// One group: problems `ids` (all of dimension d).
int run_group(kmgb_problem* pr, const std::vector<int>& ids, int d, const kmgb_options& o,
              cudaStream_t s, unsigned long long* reranked, double* loop_ms, double* phase_ms,
              Fail& f, long long* graph_launches, unsigned long long* audit) {
  const int P = (int)ids.size();
  const long long ldx = rup(d, 4);
  const long long ldb = rup(d, 8);
  const int max_iters = std::max(0, o.max_iters);
  // tensor-core tiers: a problem's rows fill whole 256-row pair units and its centers whole
  // 256-center chunks (padding centers are NaN, which the center preparation marks unusable)
  const bool tc = o.assign_tier != KMGB_ASSIGN_FP32;
  const bool split = o.assign_tier == KMGB_ASSIGN_BF16X3;
  const long long row_pad = tc ? 256 : kTileRows;
  const long long cen_pad = tc ? 256 : 1;
  // layout
  std::vector<long long> rbeg(P), rend(P), hoff(P);
  std::vector<int> coff(P), kk(P), nt(P);
  long long rows = 0, nvalid = 0, hist = 0, stiles = 0;
  long long K = 0;
  for (int i = 0; i < P; ++i) {
    const kmgb_problem& q = pr[ids[i]];
    rbeg[i] = rows;
    rend[i] = rows + q.n;
    rows += rup(q.n, row_pad);
    nvalid += q.n;
    coff[i] = (int)K;
    kk[i] = q.k;
    const long long kspan = rup(q.k, cen_pad);  // the problem's centers plus padding
    K += kspan;
    nt[i] = (int)((q.n + kSortTile - 1) / kSortTile);
    hoff[i] = hist;
    hist += kspan * nt[i];
    stiles += nt[i];
  }
  const long long tiles = rows / kTileRows;
  std::vector<int> tile_prob(tiles), stile_prob(stiles), stile_local(stiles), cprob(K);
  std::vector<int> unit_prob(tc ? rows / 256 : 0);
  for (int i = 0, st = 0; i < P; ++i) {
    const long long span = rup(rend[i] - rbeg[i], row_pad);
    for (long long t = rbeg[i] / kTileRows; t < (rbeg[i] + span) / kTileRows; ++t) tile_prob[t] = i;
    if (tc)
      for (long long u = rbeg[i] / 256; u < (rbeg[i] + span) / 256; ++u) unit_prob[u] = i;
    for (int t = 0; t < nt[i]; ++t, ++st) {
      stile_prob[st] = i;
      stile_local[st] = t;
    }
  }
  for (int i = 0; i < P; ++i) {
    const long long c1 = (i + 1 < P) ? coff[i + 1] : K;
    for (long long j = coff[i]; j < c1; ++j) cprob[j] = i;
  }
  // initial centers; padding centers are NaN (unusable, never a label, never updated)
  std::vector<float> C0((size_t)K * d, std::numeric_limits<float>::quiet_NaN());
  if (!initial_centers(pr, ids, d, C0, coff, f)) return f.code;

  DevPool m;
  const int E = KMEANS_ERROR_BUILDDATA;
  float *X = nullptr, *xn = nullptr, *C = nullptr, *Cop = nullptr, *cn = nullptr, *cmax = nullptr;
  double* qn = nullptr;
  int *labels = nullptr, *rr_list = nullptr, *rr_count = nullptr, *err = nullptr;
  unsigned long long* rr_stats = nullptr;
  // flagged rows' FP32 bands as candidates for the candidate resolve (FP32, then float-float,
  // FP64 only on near ties); rows past the capacity or with too many candidates take the exact
  // grouped pass (FP32 band, then FP64)
  const long long cand_cap = std::min<long long>(nvalid, 1LL << 20);
  int *cand = nullptr, *cand_cnt = nullptr, *rr_over = nullptr, *over_count = nullptr;
  // label audit (certified runs): KMGB_AUDIT_ROWS sampled rows (default 64) per iteration, each
  // against its own problem's centers
  int audit_rows = 0;
  if (o.certify) {
    long long ar = 64;
    if (const char* e = std::getenv("KMGB_AUDIT_ROWS")) ar = std::atoll(e);
    audit_rows = (int)std::max(0LL, std::min<long long>(ar, kAuditMaxRows));
  }
  unsigned long long* audit_ws = nullptr;
  if (f.set(m.alloc(&X, (size_t)rows * ldx), E, "data") ||
      f.set(cudaMemsetAsync(X, 0, sizeof(float) * (size_t)rows * ldx, s), E, "data") ||
      f.set(m.alloc(&xn, rows), E, "norms") || f.set(m.alloc(&qn, rows), E, "norms") ||
      f.set(m.alloc(&C, (size_t)K * ldx), E, "centers") ||
      f.set(m.alloc(&Cop, (size_t)K * ldx), E, "centers") || f.set(m.alloc(&cn, K), E, "centers") ||
      f.set(m.alloc(&cmax, 1), E, "centers") || f.set(m.alloc(&labels, rows), E, "labels") ||
      f.set(m.alloc(&rr_list, nvalid), E, "re-rank") || f.set(m.alloc(&rr_count, 1), E, "re-rank") ||
      f.set(m.alloc(&rr_stats, 2), E, "re-rank") || f.set(m.alloc(&err, 1), E, "error word") ||
      f.set(m.alloc(&cand, (size_t)cand_cap * kMaxCand), E, "re-rank") ||
      f.set(m.alloc(&cand_cnt, cand_cap), E, "re-rank") ||
      f.set(m.alloc(&rr_over, cand_cap), E, "re-rank") ||
      f.set(m.alloc(&over_count, 1), E, "re-rank") ||
      f.set(m.alloc(&audit_ws, 4 + 2 * (size_t)kAuditMaxRows), E, "audit") ||
      f.set(cudaMemsetAsync(audit_ws, 0, sizeof(unsigned long long) * (4 + 2 * kAuditMaxRows), s),
            E, "audit") ||
      f.set(cudaMemsetAsync(rr_stats, 0, 2 * sizeof(unsigned long long), s), E, "re-rank") ||
      f.set(cudaMemsetAsync(err, 0, sizeof(int), s), E, "error word") ||
      f.set(cudaMemsetAsync(C, 0, sizeof(float) * (size_t)K * ldx, s), E, "centers"))
    return f.code;
  // tensor-core tiers: BF16 planes of the points and centers, the centers' start values
  void *Xb = nullptr, *Xl = nullptr, *Cb = nullptr, *Cl = nullptr, *cbias = nullptr;
  float* cinit = nullptr;
  int* d_unit_prob = nullptr;
  if (tc &&
      (f.set(m.alloc(reinterpret_cast<uint16_t**>(&Xb), (size_t)rows * ldb), E, "BF16 data") ||
       (split && f.set(m.alloc(reinterpret_cast<uint16_t**>(&Xl), (size_t)rows * ldb), E,
                       "BF16 data")) ||
       f.set(m.alloc(reinterpret_cast<uint16_t**>(&Cb), (size_t)K * ldb), E, "BF16 centers") ||
       (split && f.set(m.alloc(reinterpret_cast<uint16_t**>(&Cl), (size_t)K * ldb), E,
                       "BF16 centers")) ||
       f.set(m.alloc(&cinit, (size_t)rup(K, kCenterPad)), E, "BF16 centers") ||
       f.set(m.alloc(reinterpret_cast<uint16_t**>(&cbias), (size_t)rup(K, kCenterPad) * kBiasCols),
             E, "BF16 centers") ||
       f.set(m.upload(&d_unit_prob, unit_prob, s), E, "tables")))
    return f.code;
  // data: host problems are packed by host threads into two pinned staging buffers in the
  // device layout (rows of ldx floats, zero padding rows and columns) while the previous buffer
  // is copied; device problems are copied on the device
  std::vector<char> is_dev(P);
  bool any_host = false;
  for (int i = 0; i < P; ++i) {
    is_dev[i] = on_device(pr[ids[i]].X) ? 1 : 0;
    any_host |= !is_dev[i];
  }
  if (any_host && !upload_host_rows(pr, ids, d, ldx, rows, row_pad, rbeg, rend, is_dev, X, s, f))
    return f.code;
  for (int i = 0; i < P; ++i) {
    const kmgb_problem& q = pr[ids[i]];
    if (is_dev[i] &&
        f.set(cudaMemcpy2DAsync(X + (size_t)rbeg[i] * ldx, sizeof(float) * ldx, q.X,
                                sizeof(float) * d, sizeof(float) * d, q.n,
                                cudaMemcpyDeviceToDevice, s),
              E, "data copy"))
      return f.code;
  }
  if (f.set(cudaMemcpy2DAsync(C, sizeof(float) * ldx, C0.data(), sizeof(float) * d,
                              sizeof(float) * d, K, cudaMemcpyHostToDevice, s),
            KMEANS_ERROR_INITIALIZE, "initial centers"))
    return f.code;
  if (f.set(launch_point_norms(X, ldx, rows, d, qn, xn, s), E, "norms")) return f.code;
  if (tc) {
    // every x a BF16 number: the split tier drops the residual plane's product
    int* inexact = nullptr;
    int host_inexact = 1;
    if (f.set(m.alloc(&inexact, 1), E, "BF16 data") ||
        f.set(cudaMemsetAsync(inexact, 0, sizeof(int), s), E, "BF16 data") ||
        f.set(launch_to_bf16(X, ldx, rows, d, Xb, ldb, s, nullptr, Xl, inexact), E, "BF16 data") ||
        f.set(cudaMemcpyAsync(&host_inexact, inexact, sizeof(int), cudaMemcpyDeviceToHost, s), E,
              "BF16 data") ||
        f.set(cudaStreamSynchronize(s), E, "BF16 data"))
      return f.code;
    if (split && host_inexact == 0) Xl = nullptr;
  }

  // problem tables
  GroupArgs g{};
  BatchUpdate b{};
  int *d_tile_prob = nullptr, *d_coff = nullptr, *d_k = nullptr, *d_nt = nullptr,
      *d_cprob = nullptr, *d_sprob = nullptr, *d_slocal = nullptr, *d_done = nullptr,
      *d_iters = nullptr;
  long long *d_rbeg = nullptr, *d_rend = nullptr, *d_hoff = nullptr;
  double *d_prev = nullptr, *d_rel = nullptr, *d_hist = nullptr;
  const int EU = KMEANS_ERROR_CLUSTER_CENTERS;
  if (f.set(m.upload(&d_tile_prob, tile_prob, s), E, "tables") ||
      f.set(m.upload(&d_coff, coff, s), E, "tables") || f.set(m.upload(&d_k, kk, s), E, "tables") ||
      f.set(m.upload(&d_nt, nt, s), E, "tables") || f.set(m.upload(&d_cprob, cprob, s), E, "tables") ||
      f.set(m.upload(&d_sprob, stile_prob, s), E, "tables") ||
      f.set(m.upload(&d_slocal, stile_local, s), E, "tables") ||
      f.set(m.upload(&d_rbeg, rbeg, s), E, "tables") || f.set(m.upload(&d_rend, rend, s), E, "tables") ||
      f.set(m.upload(&d_hoff, hoff, s), E, "tables") || f.set(m.alloc(&d_done, P), E, "tables") ||
      f.set(m.alloc(&d_iters, P), E, "tables") || f.set(m.alloc(&d_prev, P), E, "tables") ||
      f.set(m.upload(&d_rel, std::vector<double>(P, 1.0), s), E, "tables") ||
      f.set(m.alloc(&d_hist, (size_t)P * std::max(1, max_iters)), E, "tables") ||
      f.set(cudaMemsetAsync(d_done, 0, sizeof(int) * P, s), E, "tables") ||
      f.set(cudaMemsetAsync(d_iters, 0, sizeof(int) * P, s), E, "tables") ||
      f.set(cudaMemsetAsync(d_prev, 0, sizeof(double) * P, s), E, "tables"))
    return f.code;
  g.tile_prob = d_tile_prob;
  g.c_off = d_coff;
  g.k = d_k;
  g.row_end = d_rend;
  g.done = d_done;
  b.P = P;
  b.K = (int)K;
  b.n_valid = nvalid;
  b.row_beg = d_rbeg;
  b.row_end = d_rend;
  b.c_off = d_coff;
  b.k = d_k;
  b.hoff = d_hoff;
  b.ntiles = d_nt;
  b.cprob = d_cprob;
  b.stiles = stiles;
  b.stile_prob = d_sprob;
  b.stile_local = d_slocal;
  b.tile_pts = kSortTile;
  b.kmax = *std::max_element(kk.begin(), kk.end());
  b.hist_elems = hist;
  b.done = d_done;
  b.sse_prev = d_prev;
  b.rel = d_rel;
  b.iters = d_iters;
  b.sse_hist = d_hist;
  b.max_iters = std::max(1, max_iters);
  b.criterion = o.criterion;

  UpdateWork w{};
  w.n = nvalid;
  w.k = (int)K;
  w.d = d;
  w.ldx = ldx;
  w.max_pieces = nvalid / kSumPiece + K + 1;
  w.err = err;
  if (f.set(m.alloc(&w.hist, hist), EU, "update") ||
      f.set(m.alloc(&w.scan_tmp, update_scan_tmp_elems(std::max<long long>(hist, K + 1))), EU,
            "update") ||
      f.set(m.alloc(&w.label_off, K + 1), EU, "update") ||
      f.set(m.alloc(&w.piece_cnt, K + 1), EU, "update") ||
      f.set(m.alloc(&w.sorted, nvalid), EU, "update") ||
      f.set(m.alloc(&w.part, (size_t)w.max_pieces * d), EU, "update") ||
      f.set(m.alloc(&w.partq, w.max_pieces), EU, "update") ||
      f.set(m.alloc(&w.sse_k, (size_t)K * ((d + 31) / 32)), EU, "update") ||
      f.set(m.alloc(&w.counts, K), EU, "update"))
    return f.code;

  AssignArgs a{};
  a.cn = cn;
  a.xnorm = xn;
  a.cmax = cmax;
  a.labels = labels;
  a.rerank_list = rr_list;
  a.rerank_count = rr_count;
  a.err = err;
  a.n = rows;
  a.k = (int)K;
  a.d = d;
  a.certify = o.certify ? 1 : 0;
  a.gamma = tc ? assign_bf16_gamma(d) : assign_fp32_gamma(d);
  if (tc) {
    a.cinit = cinit;
    a.cbias = cbias;  // start values by MMA; padding blocks of a problem's last chunk are skipped
    a.u_prob = d_unit_prob;
    a.g_coff = d_coff;
    a.g_k = d_k;
    a.g_rend = d_rend;
    a.g_done = d_done;
  }
  RerankArgs ra{};
  ra.X = X;
  ra.ldx = ldx;
  ra.C = Cop;
  ra.ldc = ldx;
  ra.cn = cn;
  ra.list = rr_list;
  ra.count = rr_count;
  ra.labels = labels;
  ra.stats = rr_stats;
  ra.n = rows;
  ra.k = (int)K;
  ra.d = d;
  ra.mode = 0;
  ra.max_list = nvalid;
  RerankArgs rx = ra;  // the exact pass over what the candidate resolve left
  rx.list = rr_over;
  rx.count = over_count;
  rx.max_list = cand_cap;
  rx.stats = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  if (f.set(cudaEventCreate(&ev[0]), EU, "events") || f.set(cudaEventCreate(&ev[1]), EU, "events") ||
      f.set(cudaEventRecord(ev[0], s), EU, "events")) {
    for (cudaEvent_t e : ev)
      if (e) cudaEventDestroy(e);
    return f.code;
  }
  struct EvGuard {
    cudaEvent_t* e;
    ~EvGuard() {
      cudaEventDestroy(e[0]);
      cudaEventDestroy(e[1]);
    }
  } ev_guard{ev};
  // phase events of every iteration: centers | assignment | re-rank | update
  std::vector<cudaEvent_t> pev;
  struct PevGuard {
    std::vector<cudaEvent_t>* v;
    ~PevGuard() {
      for (cudaEvent_t e : *v) cudaEventDestroy(e);
    }
  } pev_guard{&pev};
  auto mark = [&]() -> bool {
    cudaEvent_t e = nullptr;
    if (f.set(cudaEventCreate(&e), EU, "events")) return false;
    pev.push_back(e);
    return !f.set(cudaEventRecord(e, s), EU, "events");
  };
  // One iteration of the group. Its launches do not depend on the iteration index (every
  // problem's SSE slot is its own device-side count), so with graphs on it is captured once and
  // replayed; phase events (marks) are recorded only in kernel-by-kernel runs.
  auto issue = [&](bool marks) -> bool {
    auto mk = [&]() { return !marks || mark(); };
    return mk() && !f.set(cudaMemsetAsync(cmax, 0, sizeof(float), s), EU, "centers") &&
           !f.set(launch_prep_centers(C, ldx, (int)K, d, Cop, Cb, ldb, cn, cmax, s, nullptr,
                                      cinit, Cl, cbias),
                  EU, "center preparation") &&
           !f.set(cudaMemsetAsync(rr_count, 0, sizeof(int), s), KMEANS_ERROR_CLOSEST_CENTERS,
                  "re-rank") &&
           mk() &&
           !f.set(tc ? launch_assign_bf16(Xb, Xl, ldb, Cb, Cl, ldb, a, s)
                     : launch_assign_fp32(X, ldx, Cop, ldx, a, s, &g, tiles),
                  KMEANS_ERROR_CLOSEST_CENTERS, "assignment") &&
           mk() &&
           !(o.certify &&
             (f.set(cudaMemsetAsync(over_count, 0, sizeof(int), s), KMEANS_ERROR_CLOSEST_CENTERS,
                    "re-rank") ||
              f.set(launch_rerank_grouped(ra, g, s, cand, cand_cnt, cand_cap),
                    KMEANS_ERROR_CLOSEST_CENTERS, "re-rank") ||
              f.set(launch_resolve_candidates(rr_list, rr_count, cand_cap, cand, cand_cnt, X, ldx,
                                              Cop, ldx, cn, d, labels, rr_over, over_count,
                                              nullptr, s),
                    KMEANS_ERROR_CLOSEST_CENTERS, "re-rank") ||
              f.set(launch_rerank_grouped(rx, g, s), KMEANS_ERROR_CLOSEST_CENTERS, "re-rank"))) &&
           !(audit_rows > 0 &&
             f.set(launch_audit_labels(X, ldx, rows, d, C, ldx, (int)K, labels, audit_ws,
                                       audit_rows, nullptr, s, &g),
                   KMEANS_ERROR_CLOSEST_CENTERS, "audit")) &&
           mk() &&
           !f.set(launch_update_batched(X, ldx, d, qn, labels, C, ldx, o.empty_policy, w, b, s),
                  EU, "update") &&
           mk();
  };
  cudaGraphExec_t gexec = nullptr;
  long long g_launches = 0;
  struct GraphGuard {
    cudaGraphExec_t* e;
    ~GraphGuard() {
      if (*e) cudaGraphExecDestroy(*e);
    }
  } graph_guard{&gexec};
  const char* gv = std::getenv("KMGB_GRAPHS");
  if (max_iters > 0 && !(gv && std::strcmp(gv, "0") == 0) &&
      cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
    const long long l0 = launch_count();
    const bool ok = issue(false);
    cudaGraph_t graph = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(s, &graph);
    g_launches = launch_count() - l0;
    count_launches(-g_launches);  // recorded into the graph, not launched
    if (ok && ec == cudaSuccess && graph &&
        cudaGraphInstantiate(&gexec, graph, 0) == cudaSuccess) {
      // captured
    } else {
      gexec = nullptr;
      cudaGetLastError();
      f.code = 0;  // a capture that failed leaves the kernel-by-kernel launches below
      f.msg.clear();
    }
    if (graph) cudaGraphDestroy(graph);
  } else {
    cudaGetLastError();
  }
  for (int it = 0; it < max_iters; ++it) {
    if (gexec) {
      if (f.set(cudaGraphLaunch(gexec, s), EU, "iteration graph")) return f.code;
      count_launches(g_launches);
      ++*graph_launches;
    } else if (!issue(true)) {
      return f.code;
    }
    if (o.criterion >= 0.0) {  // stop early once every problem's rule has fired
      std::vector<int> done(P);
      if (f.set(cudaMemcpyAsync(done.data(), d_done, sizeof(int) * P, cudaMemcpyDeviceToHost, s),
                EU, "stop flags") ||
          f.set(cudaStreamSynchronize(s), EU, "stop flags"))
        return f.code;
      if (std::all_of(done.begin(), done.end(), [](int v) { return v != 0; })) break;
    }
  }
  float ms = 0.f;
  if (f.set(cudaEventRecord(ev[1], s), EU, "events") ||
      f.set(cudaEventSynchronize(ev[1]), EU, "events") ||
      f.set(cudaEventElapsedTime(&ms, ev[0], ev[1]), EU, "events"))
    return f.code;
  *loop_ms += ms;
  for (size_t e = 0; e + 5 <= pev.size(); e += 5)  // five events per iteration
    for (int ph = 0; ph < 4; ++ph) {
      float t = 0.f;
      if (cudaEventElapsedTime(&t, pev[e + ph], pev[e + ph + 1]) == cudaSuccess) phase_ms[ph] += t;
    }
  // results
  std::vector<int> lab(rows), iters(P);
  std::vector<float> Ch((size_t)K * d);
  std::vector<double> rel(P), sh((size_t)P * std::max(1, max_iters));
  int e = 0;
  const int EG = KMEANS_ERROR_GET_CENTERS;
  if (f.set(cudaMemcpyAsync(lab.data(), labels, sizeof(int) * rows, cudaMemcpyDeviceToHost, s), EG,
            "labels") ||
      f.set(cudaMemcpy2DAsync(Ch.data(), sizeof(float) * d, C, sizeof(float) * ldx,
                              sizeof(float) * d, K, cudaMemcpyDeviceToHost, s),
            EG, "centers") ||
      f.set(cudaMemcpyAsync(iters.data(), d_iters, sizeof(int) * P, cudaMemcpyDeviceToHost, s), EG,
            "iterations") ||
      f.set(cudaMemcpyAsync(rel.data(), d_rel, sizeof(double) * P, cudaMemcpyDeviceToHost, s), EG,
            "relErr") ||
      f.set(cudaMemcpyAsync(sh.data(), d_hist, sizeof(double) * sh.size(), cudaMemcpyDeviceToHost,
                            s),
            EG, "SSE") ||
      f.set(cudaMemcpyAsync(&e, err, sizeof(int), cudaMemcpyDeviceToHost, s), EG, "error word") ||
      f.set(cudaStreamSynchronize(s), EG, "results"))
    return f.code;
  unsigned long long rs[2] = {0, 0}, au[2] = {0, 0};
  if (f.set(cudaMemcpy(rs, rr_stats, sizeof(rs), cudaMemcpyDeviceToHost), EG, "statistics") ||
      f.set(cudaMemcpy(au, audit_ws, sizeof(au), cudaMemcpyDeviceToHost), EG, "statistics"))
    return f.code;
  *reranked += rs[0];
  audit[0] += au[0];
  audit[1] += au[1];
  if (e) {
    f.code = e == KMGB_DEV_BAD_LABEL ? KMEANS_ERROR_CLUSTER_CENTERS : KMEANS_ERROR_CLOSEST_CENTERS;
    f.msg = "kmgb_lloyd_batched_f32: device error word " + std::to_string(e);
    return f.code;
  }
  for (int i = 0; i < P; ++i) {
    kmgb_problem& q = pr[ids[i]];
    if (q.labels)
      for (long long r = 0; r < q.n; ++r) q.labels[r] = lab[rbeg[i] + r] - coff[i];
    if (q.centers) std::memcpy(q.centers, Ch.data() + (size_t)coff[i] * d, sizeof(float) * q.k * d);
    q.iterations = iters[i];
    if (q.sse)
      for (int t = 0; t < iters[i]; ++t) q.sse[t] = sh[(size_t)i * b.max_iters + t];
    // kmeans.hpp:198-200: success only when relErr (1 before the first iteration) <= criterion
    q.status = (rel[i] <= o.criterion) ? KMEANS_SUCCESS : KMEANS_NONCONVERGENCE;
  }
  return 0;
}

}  // namespace

extern "C" int kmgb_lloyd_batched_f32(kmgb_problem* problems, int count, const kmgb_options* opt,
                                      kmgb_stats* stats) {
  const auto t0 = std::chrono::steady_clock::now();
  kmgb_options o;
  if (opt) o = *opt;
  else kmgb_default_options(&o);
  auto reject = [](int code, const char* msg) {
    set_last_error(msg);
    return code;
  };
  if (!problems || count <= 0) return reject(KMEANS_ERROR_BUILDDATA, "kmgb_lloyd_batched_f32: no problems");
  if (o.mini_batch_fraction < 1.0f || o.stream_tile_rows > 0 ||
      o.init_algorithm == KMGB_INIT_KMEANSPP)
    return reject(KMEANS_ERROR_BUILDDATA,
                  "kmgb_lloyd_batched_f32: batched problems use full batches, resident data and "
                  "the reference or given initialisation");
  for (int i = 0; i < count; ++i) {
    const kmgb_problem& q = problems[i];
    if (!q.X || q.n <= 0 || q.d <= 0 || q.k <= 0 || q.n >= kMaxRows || q.k > (1 << 24))
      return reject(KMEANS_ERROR_BUILDDATA,
                    "kmgb_lloyd_batched_f32: every problem needs X, 0 < n < 2^30, d > 0, k > 0");
    if (!q.init && q.k > q.n)
      return reject(KMEANS_ERROR_INITIALIZE,
                    "kmgb_lloyd_batched_f32: the reference initialisation needs k <= n");
    if (o.assign_tier == KMGB_ASSIGN_FP8)
      return reject(KMEANS_ERROR_BUILDDATA,
                    "kmgb_lloyd_batched_f32: the FP8 tier runs single problems only");
    if (o.assign_tier != KMGB_ASSIGN_FP32 && o.assign_tier != KMGB_ASSIGN_AUTO &&
        !bf16_tc_supported(q.d, o.assign_tier == KMGB_ASSIGN_BF16X3 ? 2 : 1))
      return reject(KMEANS_ERROR_BUILDDATA,
                    "kmgb_lloyd_batched_f32: the BF16 tensor-core tiers support D <= 512 "
                    "(320 for the split tier)");
  }
  for (int i = 0; i < count; ++i) {
    problems[i].iterations = 0;
    problems[i].status = KMEANS_NONCONVERGENCE;
  }
  // groups: problems of one dimension and tier, split so that every group fits the index and
  // scan limits
  std::vector<int> order(count), ptier = tiers_of(o, problems, count);
  for (int i = 0; i < count; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    return problems[x].d != problems[y].d ? problems[x].d < problems[y].d : ptier[x] < ptier[y];
  });
  cudaStream_t s = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess)
    return reject(KMEANS_ERROR_BUILDDATA, "kmgb_lloyd_batched_f32: stream creation failed");
  Fail f;
  unsigned long long reranked = 0, audit[2] = {0, 0};  // audit: rows audited, violations
  double loop_ms = 0.0;
  double phase_ms[4] = {0.0, 0.0, 0.0, 0.0};
  long long graph_launches = 0;
  size_t i = 0;
  long long groups = 0;
  while (i < order.size() && !f.code) {
    const int d = problems[order[i]].d;
    const int tier = ptier[order[i]];
    const bool tc = tier != KMGB_ASSIGN_FP32;
    const long long row_pad = tc ? 256 : kTileRows, cen_pad = tc ? 256 : 1;
    const long long ldx = rup(d, 4);
    std::vector<int> ids;
    long long rows = 0, hist = 0, K = 0;
    while (i < order.size() && problems[order[i]].d == d && ptier[order[i]] == tier) {
      const kmgb_problem& q = problems[order[i]];
      const long long r = rup(q.n, row_pad);
      const long long kspan = rup(q.k, cen_pad);
      const long long h = kspan * ((q.n + kSortTile - 1) / kSortTile);
      if (!ids.empty() && (rows + r > kMaxRows || hist + h > kMaxHist || K + kspan > (1LL << 30) ||
                           (rows + r) * ldx * 4 > kMaxXBytes))
        break;
      if (h > kMaxHist) {
        f.code = KMEANS_ERROR_BUILDDATA;
        f.msg = "kmgb_lloyd_batched_f32: a problem's k x ceil(n/2048) exceeds the sort capacity";
        break;
      }
      ids.push_back(order[i]);
      rows += r;
      hist += h;
      K += kspan;
      ++i;
    }
    if (f.code) break;
    kmgb_options og = o;
    og.assign_tier = tier;
    run_group(problems, ids, d, og, s, &reranked, &loop_ms, phase_ms, f, &graph_launches, audit);
    ++groups;
  }
  cudaStreamSynchronize(s);
  cudaStreamDestroy(s);
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    int it = 0;
    for (int j = 0; j < count; ++j) it = std::max(it, problems[j].iterations);
    stats->iterations = it;
    stats->status = f.code;
    stats->reranked = reranked;
    stats->ms_total = loop_ms;
    // reserved[1..4]: microseconds of center preparation, assignment, re-rank and update
    for (int ph = 0; ph < 4; ++ph) stats->reserved[1 + ph] = (long long)(phase_ms[ph] * 1000.0);
    stats->reserved[5] = graph_launches;
    stats->reserved[6] = groups;
    // rows audited against the FP64 arg-min over their problem's centers (high 40 bits) and
    // violations found (low 24 bits, saturating)
    stats->reserved[7] = (long long)((audit[0] << 24) | std::min<unsigned long long>(audit[1], 0xFFFFFF));
    stats->reserved[0] = (long long)std::chrono::duration<double, std::micro>(
                             std::chrono::steady_clock::now() - t0)
                             .count();
  }
  if (f.code) {
    set_last_error(f.msg.c_str());
    return f.code;
  }
  return 0;
}
