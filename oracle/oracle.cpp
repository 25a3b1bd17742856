// Oracle for the K-means Lloyd hot path -- TEST INFRASTRUCTURE ONLY.
//
// This file is a CPU restatement of the reference algorithm (PaulMullowney/kmeans) used by
// tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the checker. The
// product library (kmeans_gb300/) never links, loads or calls it.
//
// Parity status: the reference has no CPU path and ships no golden vectors. The oracle is
// pinned (1) to the reference's own known-answer procedure (test/python/distance.py.in:75-79,
// arg-min of the norm expansion with numpy) and to independent restatements of its host-side
// random streams through the committed fixtures in tests/golden/, and (2) to the reference's
// own kernels (main/cuda/ClosestCenters.cu, ClusterCenters.cu and Compactness.cu built from its
// sources for the GPU and launched with its grids; tests/test_gpu_reference_kernels.py): their
// labels equal the oracle's on the test mixtures, their centers are within the FP32 error bound
// of the oracle's exact means (NaN for empty clusters in both) and their compactness within
// the FP32 bound of the oracle's SSE. The reference's host loop is not run; its rules follow
// its source line by line as cited below.
//
// Semantics restated here:
//  * shuffle   : std::shuffle of row indices with std::default_random_engine(0)
//                (main/cpp/kmeans.cpp:554-564). perm[i] = source row of shuffled row i.
//  * init      : srand(42); index = rand() % m, re-drawn while binary_search() on the
//                UNSORTED pick list finds it (kmeans.cpp:876-883). Center i = shuffled row
//                picks[i] (kmeans.cpp:886-888).
//  * assignment: label = arg-min over centers of the squared distance, lowest index on ties
//                (ClosestCenters.cu:105-123 strict '<' across blocks, reduction.hcu:60-64,
//                RowTransformMinimum.cu:43-50). Here the distance is evaluated exactly as
//                an FP64 fma chain sum_d ((double)x_d - (double)c_d)^2, so the oracle label
//                is the FP64 arg-min. NaN centers (empty clusters) never win, as in
//                RowTransformMinimum.cu:31 ('val<dataReg' is false for NaN).
//  * update    : new center = sum of member points / count (ClusterCenters.cu:3-23,47-87);
//                count 0 gives 0/0 = NaN (ClusterCenters.cu:81) under the reference policy.
//                Sums in a canonical order: members in ascending point order, grouped in
//                pieces of `piece` points; each piece is summed from zero (FP32 data: an
//                error-free float-float TwoSum, ~48 bits, converted to FP64 once; FP64 data:
//                FP64), pieces are summed in order in FP64; the quotient is rounded once.
//  * SSE       : sum_i ||x_i - c_new[label_i]||^2 against the NEW centers with the labels of
//                the OLD centers (Compactness.cu:3-59, kmeans.cpp:1044-1104), FP64.
//  * loop      : while (iters < maxIters && relErr > criterion), relErr =
//                |SSE - SSE_old| / |SSE| with SSE_old = 0 initially (kmeans.cpp:1194-1240);
//                status 13 (KMEANS_NONCONVERGENCE) when relErr > criterion at exit
//                (kmeans.hpp:198-200).
//  * mini-batch: m_mb = (int)(fraction * m) in float arithmetic (kmeans.cpp:79); iteration t
//                uses shuffled rows [(t*m_mb) mod m, +m_mb) with wrap-around
//                (kmeans.cpp:426-447, 746-753, 801-808); the new centers are the means of
//                that window only and SSE is that window's (kmeans.cpp:1050-1060, 1252-1312).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <random>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

template <typename T>
inline double dist64(const T* x, const T* c, int d) {
  double s = 0.0;
  for (int t = 0; t < d; ++t) {
    double u = (double)x[t] - (double)c[t];
    s = std::fma(u, u, s);
  }
  return s;
}

// Rows of the window used by iteration `it` (shuffled order mapped to source rows).
void window_rows(const int* perm, long long m, long long m_mb, int it, std::vector<long long>& rows) {
  rows.resize(m_mb);
  long long start = 0;
  // Incremental wrap exactly as kmeans.cpp:428-441 (mCurrent += m_mb; wrap when > m, == m -> 0).
  for (int t = 0; t < it; ++t) {
    start += m_mb;
    if (start > m) start = start % m;
    else if (start == m) start = 0;
  }
  for (long long r = 0; r < m_mb; ++r) {
    long long pos = start + r;
    if (pos >= m) pos -= m;
    rows[r] = perm[pos];
  }
}

}  // namespace

extern "C" {

// std::shuffle with default_random_engine(0) over 0..m-1 (kmeans.cpp:554-557).
void orc_shuffle_perm(int m, int* perm) {
  std::vector<int> idx(m);
  for (int i = 0; i < m; ++i) idx[i] = i;
  unsigned seed = 0;
  std::shuffle(idx.begin(), idx.end(), std::default_random_engine(seed));
  std::memcpy(perm, idx.data(), sizeof(int) * (size_t)m);
}

// srand(42) / rand() % m picks with the reference's binary_search on an unsorted vector
// (kmeans.cpp:876-883). glibc's random_r with a private TYPE_3 state seeded with 42 gives the
// same stream as srand(42)/rand() without touching the process-wide generator.
int orc_init_picks(int m, int k, int* picks) {
  if (m <= 0 || k <= 0 || k > m) return -1;
  struct random_data rd;
  std::memset(&rd, 0, sizeof(rd));
  static char state[128];
  std::memset(state, 0, sizeof(state));
  if (initstate_r(42u, state, sizeof(state), &rd) != 0) return -2;
  std::vector<int> points;
  points.reserve(k);
  for (int i = 0; i < k; ++i) {
    int32_t r = 0;
    random_r(&rd, &r);
    int index = r % m;
    while (std::binary_search(points.begin(), points.end(), index)) {
      random_r(&rd, &r);
      index = r % m;
    }
    points.push_back(index);
  }
  std::memcpy(picks, points.data(), sizeof(int) * (size_t)k);
  return 0;
}

// Reference initial centers, K x D row-major: center i = shuffled row picks[i].
int orc_reference_init(const float* X, int m, int d, int k, float* centers) {
  std::vector<int> perm(m), picks(k);
  orc_shuffle_perm(m, perm.data());
  int rc = orc_init_picks(m, k, picks.data());
  if (rc) return rc;
  for (int i = 0; i < k; ++i)
    std::memcpy(centers + (size_t)i * d, X + (size_t)perm[picks[i]] * d, sizeof(float) * d);
  return 0;
}

}  // extern "C"

// FP64 arg-min labels over `rows` (nullptr = all rows 0..m-1). best_out (nullable) gets the
// FP64 distance of the chosen center.
template <typename T>
void assign_rows(const T* X, long long nrows, const long long* rows, int d, const T* C, int k,
                 int* labels, double* best_out) {
#pragma omp parallel for schedule(static)
  for (long long r = 0; r < nrows; ++r) {
    const long long i = rows ? rows[r] : r;
    const T* x = X + (size_t)i * d;
    double b = std::numeric_limits<double>::infinity();
    int bi = -1;
    for (int j = 0; j < k; ++j) {
      double v = dist64(x, C + (size_t)j * d, d);
      if (v < b) { b = v; bi = j; }
    }
    if (bi < 0) bi = 0;  // no finite distance: label 0 (both sides agree on this rule)
    labels[r] = bi;
    if (best_out) best_out[r] = b;
  }
}

// Piece accumulator, the same operation sequence as the device: FP32 data are summed with an
// error-free float-float TwoSum (hi + lo), converted to FP64 once per piece; FP64 data are
// summed in FP64.
template <typename T>
struct PieceAcc;
template <>
struct PieceAcc<float> {
  float hi = 0.0f, lo = 0.0f;
  void add(float x) {
    const float t = hi + x;
    const float bp = t - hi;
    const float err = (hi - (t - bp)) + (x - bp);
    hi = t;
    lo = lo + err;
  }
  double value() const { return (double)hi + (double)lo; }
};
template <>
struct PieceAcc<double> {
  double s = 0.0;
  void add(double x) { s += x; }
  double value() const { return s; }
};

// Canonical FP64 center update over `rows` (nullptr = 0..m-1), labels indexed like rows.
// new_centers: K x D of T (the FP64 quotient rounded once to T). counts: K (nullable).
// sums: K x D FP64 (nullable). empty_policy 0: NaN center for an empty cluster (reference);
// 1: keep old center.
template <typename T>
void update_rows(const T* X, long long nrows, const long long* rows, int d, const int* labels,
                 int k, int piece, const T* old_centers, int empty_policy, T* new_centers,
                 long long* counts, double* sums) {
  std::vector<long long> cnt(k, 0);
  for (long long r = 0; r < nrows; ++r) cnt[labels[r]]++;
  std::vector<long long> off(k + 1, 0);
  for (int j = 0; j < k; ++j) off[j + 1] = off[j] + cnt[j];
  std::vector<long long> sorted(nrows);
  std::vector<long long> pos(off.begin(), off.end() - 1);
  for (long long r = 0; r < nrows; ++r) sorted[pos[labels[r]]++] = r;  // stable

#pragma omp parallel for schedule(dynamic, 1)
  for (int j = 0; j < k; ++j) {
    std::vector<double> total(d, 0.0);
    std::vector<PieceAcc<T>> part(d);
    for (long long p0 = off[j]; p0 < off[j + 1]; p0 += piece) {
      long long p1 = std::min(p0 + (long long)piece, off[j + 1]);
      std::fill(part.begin(), part.end(), PieceAcc<T>());
      for (long long q = p0; q < p1; ++q) {
        const long long r = sorted[q];
        const long long i = rows ? rows[r] : r;
        const T* x = X + (size_t)i * d;
        for (int t = 0; t < d; ++t) part[t].add(x[t]);
      }
      for (int t = 0; t < d; ++t) total[t] += part[t].value();
    }
    const long long n = cnt[j];
    for (int t = 0; t < d; ++t) {
      T v;
      if (n > 0) v = (T)(total[t] / (double)n);
      else if (empty_policy == 1 && old_centers) v = old_centers[(size_t)j * d + t];
      else v = std::numeric_limits<T>::quiet_NaN();
      new_centers[(size_t)j * d + t] = v;
      if (sums) sums[(size_t)j * d + t] = total[t];
    }
    if (counts) counts[j] = n;
  }
}

// FP64 SSE against `centers` (direct form), deterministic chunked order.
template <typename T>
double sse_rows(const T* X, long long nrows, const long long* rows, int d, const int* labels,
                const T* centers) {
  const long long CH = 4096;
  const long long nch = (nrows + CH - 1) / CH;
  std::vector<double> part(nch > 0 ? nch : 1, 0.0);
#pragma omp parallel for schedule(static)
  for (long long c = 0; c < nch; ++c) {
    double s = 0.0;
    for (long long r = c * CH; r < std::min(nrows, (c + 1) * CH); ++r) {
      const long long i = rows ? rows[r] : r;
      s += dist64(X + (size_t)i * d, centers + (size_t)labels[r] * d, d);
    }
    part[c] = s;
  }
  double t = 0.0;
  for (long long c = 0; c < nch; ++c) t += part[c];
  return t;
}

// Full Lloyd loop (full batch when mb_fraction >= 1, else the reference's mini-batch
// windows over the shuffled order). init: K x D row-major. Returns 0 (converged) or 13.
// labels_out (nullable): labels of the last assignment at source-row positions (-1 for rows
// outside the last mini-batch window). sse_out (nullable): per-iteration SSE.
template <typename T>
int lloyd(const T* X, long long m, int d, int k, const T* init, int max_iters, double criterion,
          float mb_fraction, int empty_policy, int piece, T* centers_out, int* labels_out,
          double* sse_out, int* iters_out) {
  std::vector<T> cur(init, init + (size_t)k * d), nxt((size_t)k * d);
  const bool mini = mb_fraction < 1.0f;
  long long m_mb = mini ? (long long)(int)(mb_fraction * (float)m) : m;
  std::vector<int> perm;
  if (mini) {
    perm.resize(m);
    orc_shuffle_perm((int)m, perm.data());
  }
  std::vector<long long> rows;
  std::vector<int> labels(m_mb);
  double sse_old = 0.0, rel = 1.0;
  int it = 0;
  while (it < max_iters && rel > criterion) {
    const long long* rp = nullptr;
    if (mini) {
      window_rows(perm.data(), m, m_mb, it, rows);
      rp = rows.data();
    }
    assign_rows<T>(X, m_mb, rp, d, cur.data(), k, labels.data(), nullptr);
    update_rows<T>(X, m_mb, rp, d, labels.data(), k, piece, cur.data(), empty_policy, nxt.data(),
                   nullptr, nullptr);
    double sse = sse_rows<T>(X, m_mb, rp, d, labels.data(), nxt.data());
    rel = std::fabs(sse - sse_old) / std::fabs(sse);
    sse_old = sse;
    if (sse_out) sse_out[it] = sse;
    cur.swap(nxt);
    ++it;
  }
  std::memcpy(centers_out, cur.data(), sizeof(T) * (size_t)k * d);
  if (labels_out) {
    if (mini) {
      for (long long i = 0; i < m; ++i) labels_out[i] = -1;
      for (long long r = 0; r < m_mb; ++r) labels_out[rows[r]] = labels[r];
    } else {
      std::memcpy(labels_out, labels.data(), sizeof(int) * (size_t)m);
    }
  }
  if (iters_out) *iters_out = it;
  return (rel <= criterion) ? 0 : 13;
}

// Host-streamed tiles (the reference's out-of-memory path, kmeans.cpp:301-536, 699-818, with
// one pass per iteration): rows [t*tile, (t+1)*tile) form tile t; each tile's canonical per-center
// sums (update_rows on the tile: pieces of its label-sorted members, summed from zero in piece
// order) are added to the FP64 totals one tile at a time, tiles in order; the center is the total
// over the count, rounded once.
template <typename T>
void update_tiled(const T* X, long long m, int d, const int* labels, int k, int piece,
                  long long tile, const T* old_centers, int empty_policy, T* new_centers) {
  std::vector<double> total((size_t)k * d, 0.0), sums((size_t)k * d);
  std::vector<long long> cnt(k, 0), tcnt(k);
  std::vector<T> scratch((size_t)k * d);
  for (long long r0 = 0; r0 < m; r0 += tile) {
    const long long nt = std::min(tile, m - r0);
    update_rows<T>(X + (size_t)r0 * d, nt, nullptr, d, labels + r0, k, piece, nullptr, 0,
                   scratch.data(), tcnt.data(), sums.data());
    for (size_t e = 0; e < total.size(); ++e) total[e] += sums[e];
    for (int j = 0; j < k; ++j) cnt[j] += tcnt[j];
  }
  for (int j = 0; j < k; ++j)
    for (int t = 0; t < d; ++t) {
      T v;
      if (cnt[j] > 0) v = (T)(total[(size_t)j * d + t] / (double)cnt[j]);
      else if (empty_policy == 1 && old_centers) v = old_centers[(size_t)j * d + t];
      else v = std::numeric_limits<T>::quiet_NaN();
      new_centers[(size_t)j * d + t] = v;
    }
}

// Full-batch Lloyd loop with the host-streamed tiles' update order.
template <typename T>
int lloyd_tiled(const T* X, long long m, int d, int k, const T* init, int max_iters,
                double criterion, int empty_policy, int piece, long long tile, T* centers_out,
                int* labels_out, double* sse_out, int* iters_out) {
  std::vector<T> cur(init, init + (size_t)k * d), nxt((size_t)k * d);
  std::vector<int> labels(m);
  double sse_old = 0.0, rel = 1.0;
  int it = 0;
  while (it < max_iters && rel > criterion) {
    assign_rows<T>(X, m, nullptr, d, cur.data(), k, labels.data(), nullptr);
    update_tiled<T>(X, m, d, labels.data(), k, piece, tile, cur.data(), empty_policy, nxt.data());
    const double sse = sse_rows<T>(X, m, nullptr, d, labels.data(), nxt.data());
    rel = std::fabs(sse - sse_old) / std::fabs(sse);
    sse_old = sse;
    if (sse_out) sse_out[it] = sse;
    cur.swap(nxt);
    ++it;
  }
  std::memcpy(centers_out, cur.data(), sizeof(T) * (size_t)k * d);
  if (labels_out) std::memcpy(labels_out, labels.data(), sizeof(int) * (size_t)m);
  if (iters_out) *iters_out = it;
  return (rel <= criterion) ? 0 : 13;
}

extern "C" {

int orc_lloyd_tiled(const float* X, long long m, int d, int k, const float* init, int max_iters,
                    double criterion, int empty_policy, int piece, long long tile,
                    float* centers_out, int* labels_out, double* sse_out, int* iters_out) {
  return lloyd_tiled<float>(X, m, d, k, init, max_iters, criterion, empty_policy, piece, tile,
                            centers_out, labels_out, sse_out, iters_out);
}

void orc_assign(const float* X, long long m, int d, const float* C, int k, int* labels,
                double* best_out) {
  assign_rows<float>(X, m, nullptr, d, C, k, labels, best_out);
}
void orc_assign_d(const double* X, long long m, int d, const double* C, int k, int* labels,
                  double* best_out) {
  assign_rows<double>(X, m, nullptr, d, C, k, labels, best_out);
}
void orc_update(const float* X, long long m, int d, const int* labels, int k, int piece,
                const float* old_centers, int empty_policy, float* new_centers, long long* counts,
                double* sums) {
  update_rows<float>(X, m, nullptr, d, labels, k, piece, old_centers, empty_policy, new_centers,
                     counts, sums);
}
void orc_update_d(const double* X, long long m, int d, const int* labels, int k, int piece,
                  const double* old_centers, int empty_policy, double* new_centers,
                  long long* counts, double* sums) {
  update_rows<double>(X, m, nullptr, d, labels, k, piece, old_centers, empty_policy, new_centers,
                      counts, sums);
}
double orc_sse(const float* X, long long m, int d, const int* labels, const float* centers) {
  return sse_rows<float>(X, m, nullptr, d, labels, centers);
}
double orc_sse_d(const double* X, long long m, int d, const int* labels, const double* centers) {
  return sse_rows<double>(X, m, nullptr, d, labels, centers);
}
int orc_lloyd(const float* X, long long m, int d, int k, const float* init, int max_iters,
              double criterion, float mb_fraction, int empty_policy, int piece,
              float* centers_out, int* labels_out, double* sse_out, int* iters_out) {
  return lloyd<float>(X, m, d, k, init, max_iters, criterion, mb_fraction, empty_policy, piece,
                      centers_out, labels_out, sse_out, iters_out);
}
int orc_lloyd_d(const double* X, long long m, int d, int k, const double* init, int max_iters,
                double criterion, float mb_fraction, int empty_policy, int piece,
                double* centers_out, int* labels_out, double* sse_out, int* iters_out) {
  return lloyd<double>(X, m, d, k, init, max_iters, criterion, mb_fraction, empty_policy, piece,
                       centers_out, labels_out, sse_out, iters_out);
}
// Closest centers with caller norms (per-kernel ABI, ClosestCenters.cu semantics restated in
// FP64): label = arg-min_j fma(-2, dot64(x, c_j), nb_j), lowest j on ties; B is d x k.
void orc_closest_expansion(const float* A, int m, int d, const float* B, int k,
                           const float* nb, int* labels) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < m; ++i) {
    double best = std::numeric_limits<double>::infinity();
    int bi = -1;
    for (int j = 0; j < k; ++j) {
      double s = 0.0;
      for (int t = 0; t < d; ++t) s = std::fma((double)A[(size_t)i * d + t], (double)B[(size_t)t * k + j], s);
      const double v = std::fma(-2.0, s, (double)nb[j]);
      if (v < best) { best = v; bi = j; }
    }
    labels[i] = bi < 0 ? 0 : bi;
  }
}
void orc_closest_expansion_d(const double* A, int m, int d, const double* B, int k,
                             const double* nb, int* labels) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < m; ++i) {
    double best = std::numeric_limits<double>::infinity();
    int bi = -1;
    for (int j = 0; j < k; ++j) {
      double s = 0.0;
      for (int t = 0; t < d; ++t) s = std::fma(A[(size_t)i * d + t], B[(size_t)t * k + j], s);
      const double v = std::fma(-2.0, s, nb[j]);
      if (v < best) { best = v; bi = j; }
    }
    labels[i] = bi < 0 ? 0 : bi;
  }
}

// ---- per-kernel reference entry semantics (reference layouts) ----

// rowTransformMinimum (RowTransformMinimum.cu:3-58): per row i the arg-min over j of
// normA[i] + normB[j] - 2*G[i*n+j], evaluated as the reference evaluates it for TYPE=float
// (float sum of the norms, then a double subtraction of 2.0*G, rounded back to float), strict
// '<' in column order so the lowest index wins ties; output[m0+i].
void orc_row_transform_min_f(int m0, int m, int n, const float* normA, const float* normB,
                             const float* G, int* out) {
  for (int i = 0; i < m; ++i) {
    float best = std::numeric_limits<float>::max();
    int bi = -1;
    const float a = normA[i];
    for (int j = 0; j < n; ++j) {
      float s = a + normB[j];
      float v = (float)((double)s - 2.0 * (double)G[(size_t)i * n + j]);
      if (v < best) { best = v; bi = j; }
    }
    out[m0 + i] = bi;
  }
}

void orc_row_transform_min_d(int m0, int m, int n, const double* normA, const double* normB,
                             const double* G, int* out) {
  for (int i = 0; i < m; ++i) {
    double best = std::numeric_limits<float>::max();  // FLT_MAX as in the reference
    int bi = -1;
    const double a = normA[i];
    for (int j = 0; j < n; ++j) {
      double v = a + normB[j] - 2.0 * G[(size_t)i * n + j];
      if (v < best) { best = v; bi = j; }
    }
    out[m0 + i] = bi;
  }
}

// ---- FP32 port: the CPU baseline (same loop, FP32 norm-expansion assignment) ----
// Timed on the host cores as the stand-in for the reference's (absent) CPU path. The
// assignment uses the reference's own distance form ||c||^2 - 2 x.c in FP32 with the centers
// in the reference's D x K layout (kmeans.cpp:886-888), vectorised across centers.
__attribute__((optimize("fp-contract=fast")))
static void port_assign_block(const float* X, long long i0, long long i1, int d, const float* CT,
                              const float* cn, int k, int* labels) {
  const int JB = 256;
  std::vector<float> acc((size_t)4 * JB);
  for (long long i = i0; i < i1; i += 4) {
    const int np = (int)std::min<long long>(4, i1 - i);
    float best[4];
    int bi[4];
    for (int p = 0; p < 4; ++p) { best[p] = std::numeric_limits<float>::infinity(); bi[p] = 0; }
    for (int j0 = 0; j0 < k; j0 += JB) {
      const int jn = std::min(JB, k - j0);
      std::fill(acc.begin(), acc.end(), 0.0f);
      for (int t = 0; t < d; ++t) {
        const float* crow = CT + (size_t)t * k + j0;
        for (int p = 0; p < np; ++p) {
          const float xv = X[(size_t)(i + p) * d + t];
          float* a = acc.data() + (size_t)p * JB;
          for (int j = 0; j < jn; ++j) a[j] += xv * crow[j];
        }
      }
      for (int p = 0; p < np; ++p) {
        const float* a = acc.data() + (size_t)p * JB;
        for (int j = 0; j < jn; ++j) {
          float v = cn[j0 + j] - 2.0f * a[j];
          if (v < best[p]) { best[p] = v; bi[p] = j0 + j; }
        }
      }
    }
    for (int p = 0; p < np; ++p) labels[i + p] = bi[p];
  }
}

// One or more full-batch FP32-port Lloyd iterations over rows [0, m). Returns iterations.
int orc_port_lloyd(const float* X, long long m, int d, int k, const float* init, int iters,
                   int piece, float* centers_out, int* labels_out, double* sse_out) {
  std::vector<float> cur(init, init + (size_t)k * d), nxt((size_t)k * d), CT((size_t)d * k), cn(k);
  std::vector<int> labels(m);
  for (int it = 0; it < iters; ++it) {
    for (int j = 0; j < k; ++j) {
      float s = 0.0f;
      for (int t = 0; t < d; ++t) {
        const float v = cur[(size_t)j * d + t];
        CT[(size_t)t * k + j] = v;
        s += v * v;
      }
      cn[j] = s;
    }
    const long long B = 256;
    const long long nb = (m + B - 1) / B;
#pragma omp parallel for schedule(dynamic, 4)
    for (long long b = 0; b < nb; ++b)
      port_assign_block(X, b * B, std::min(m, (b + 1) * B), d, CT.data(), cn.data(), k,
                        labels.data());
    update_rows<float>(X, m, nullptr, d, labels.data(), k, piece, cur.data(), 0, nxt.data(),
                       nullptr, nullptr);
    double sse = sse_rows<float>(X, m, nullptr, d, labels.data(), nxt.data());
    if (sse_out) sse_out[it] = sse;
    cur.swap(nxt);
  }
  std::memcpy(centers_out, cur.data(), sizeof(float) * (size_t)k * d);
  if (labels_out) std::memcpy(labels_out, labels.data(), sizeof(int) * (size_t)m);
  return iters;
}

// k-means++ initialisation restated from the library's documented draw rule (an extension: the
// reference declares initAlgorithm/numRetries, main/cpp/kmeans.hpp:94-95, and never reads them).
// D^2 per point in T: 32 lane partials (lane l takes dims l, l+32, ... as an fma chain of
// (x-c)^2), then the xor butterfly s_l += s_(l^o) for o = 16..1; D^2 = fmin over the centers
// drawn so far. Weights q = saturating truncation of D^2 * (2^31 / M) in T, M = max D^2.
// Draw r: u = splitmix64(splitmix64(seed) + r) >> 11; target = (u * sum q) >> 53; the point
// whose [prefix, prefix + q) holds target. Draw 0, or a zero total, picks (u * n) >> 53.
}  // extern "C"

namespace {

inline uint64_t orc_splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

template <typename T>
T kpp_dist(const T* x, const T* c, int d) {
  T lanes[32];
  for (int l = 0; l < 32; ++l) {
    T s = T(0);
    for (int t = l; t < d; t += 32) {
      const T u = x[t] - c[t];
      s = std::fma(u, u, s);
    }
    lanes[l] = s;
  }
  for (int o = 16; o > 0; o >>= 1) {
    T nx[32];
    for (int l = 0; l < 32; ++l) nx[l] = lanes[l] + lanes[l ^ o];
    std::memcpy(lanes, nx, sizeof(lanes));
  }
  return lanes[0];
}

template <typename T>
uint32_t kpp_weight(T v, T scale) {
  const T p = v * scale;
  if (!(p > T(0))) return 0u;  // NaN, zero
  if (p >= T(4294967296.0)) return 0xffffffffu;
  return (uint32_t)p;
}

template <typename T>
int kmeanspp(const T* X, long long n, int d, int k, unsigned long long seed, int* picks, T* centers) {
  if (n <= 0 || d <= 0 || k <= 0 || k > n) return -1;
  std::vector<T> d2(n);
  std::vector<uint32_t> q(n);
  const uint64_t s0 = orc_splitmix64(seed);
  for (int r = 0; r < k; ++r) {
    unsigned long long total = 0;
    if (r > 0) {
      const T* c = X + (size_t)picks[r - 1] * d;
      const bool first = r == 1;
#pragma omp parallel for schedule(static)
      for (long long i = 0; i < n; ++i) {
        const T s = kpp_dist(X + (size_t)i * d, c, d);
        d2[i] = first ? s : std::fmin(d2[i], s);
      }
      T M = T(0);
      for (long long i = 0; i < n; ++i)
        if (d2[i] > M) M = d2[i];
      const T scale = M > T(0) ? T(2147483648.0) / M : T(0);
      for (long long i = 0; i < n; ++i) {
        q[i] = kpp_weight(d2[i], scale);
        total += q[i];
      }
    }
    const uint64_t u = orc_splitmix64(s0 + (uint64_t)r) >> 11;
    long long chosen = (long long)(((unsigned __int128)u * (unsigned long long)n) >> 53);
    if (total > 0) {
      const unsigned long long target = (unsigned long long)(((unsigned __int128)u * total) >> 53);
      unsigned long long ex = 0;
      for (long long i = 0; i < n; ++i) {
        if (q[i] > 0 && target < ex + q[i]) {
          chosen = i;
          break;
        }
        ex += q[i];
      }
    }
    picks[r] = (int)chosen;
  }
  if (centers)
    for (int j = 0; j < k; ++j)
      std::memcpy(centers + (size_t)j * d, X + (size_t)picks[j] * d, sizeof(T) * d);
  return 0;
}

}  // namespace

extern "C" {

int orc_kmeanspp(const float* X, long long n, int d, int k, unsigned long long seed, int* picks,
                 float* centers) {
  return kmeanspp<float>(X, n, d, k, seed, picks, centers);
}

int orc_kmeanspp_d(const double* X, long long n, int d, int k, unsigned long long seed, int* picks,
                   double* centers) {
  return kmeanspp<double>(X, n, d, k, seed, picks, centers);
}

int orc_num_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
