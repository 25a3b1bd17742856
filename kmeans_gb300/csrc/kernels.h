// Internal launch interface of the GB300 Lloyd kernels (not part of the public C-ABI).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

namespace kmgb {

// Certified assignment: labels plus a list of points whose top-2 margin does not prove the
// FP64 arg-min. `gamma` is the relative error of the approximate dot product
// (|fl(x.c) - x.c| <= gamma * ||x|| * ||c||).
struct AssignArgs {
  const float* cn;        // [k] ||c_j||^2 rounded to FP32, +inf for unusable (NaN) centers
  const float* xnorm;     // [n] upper bound of ||x_i||
  const float* cmax;      // device scalar: upper bound of max ||c_j|| over usable centers
  const float* cinit;     // [round_up(k,128)] accumulator start -||c_j||^2/2 (BF16 tier)
  const void* cbias;      // nullable: the same start values as BF16 pieces (launch_prep_centers'
                          // cbias); when given, the pair kernel's first MMA of every chunk loads
                          // them into the accumulator and the epilogue adds nothing
  float* dump;            // diagnostic (nullable): raw accumulators [n][round_up(k,128)]
  // BF16 tiers only:
  const int* n_dev;       // nullable: rows actually present = min(*n_dev, n) (device count)
  long long row0;         // first row of this batch (rows row0 .. row0 + present - 1)
  long long out0;         // full pass: the launch's rows are rows out0.. of the data set (labels,
                          // norms, floors and flagged-list entries are indexed by those)
  float* thr_out;         // nullable: for every flagged point, best key - 2E (candidate floor)
  const float* thr_in;    // candidate mode: per-row floor; keys >= floor are recorded in cand
  int* cand;              // candidate mode: [n][kMaxCand] center indices
  int* cand_cnt;          // candidate mode: [n] count, -1 if more than kMaxCand
  int* labels;            // [n]
  int* rerank_list;       // [n]
  int* rerank_count;      // device scalar
  int* err;               // device error word
  long long n;
  int k;
  int d;
  int certify;            // 0: write arg-min labels only
  float gamma;
  float pert;             // FP64 data rounded to FP32 for the tensor pass: every key's bound
                          // grows by 1.02 pert (||x|| cmax 1.01 + cmax^2 / 2); 0 for FP32 data
  const int* stop;        // device stop flag of the run (nullable)
  // BF16 tiers, grouped problems (batched Lloyd; null otherwise): unit u (rows 256u .. 256u+255)
  // belongs to problem u_prob[u], whose centers are rows g_coff[p] .. g_coff[p] + g_k[p] - 1 (a
  // multiple of 256 apart, padding centers unusable); labels are global center indices; rows at
  // or past g_rend[p] are not written; units of problems with g_done[p] set are skipped
  const int* u_prob;
  const int* g_coff;
  const int* g_k;
  const long long* g_rend;
  const int* g_done;
  // BF16 tiers, store mode (the router's hidden layer; null otherwise): instead of the arg-max,
  // every key (accumulator + cinit[j]) is written as BF16 to store_out[row * store_ld + j],
  // clamped at zero when store_relu is set; labels and the certificate are not produced
  void* store_out;
  long long store_ld;
  int store_relu;
  // BF16 tiers, separation mode (the router; null otherwise): X and C are the same centers in
  // group order, every 256-row unit and 256-center chunk inside one group (slot_group[slot]);
  // for every row xmax_out receives an upper bound of the largest exact key x.c - |c|^2/2 over
  // the centers of the other groups (-inf if none), the epilogue skipping the row's own group's
  // chunks; needs cbias, no certificate, no labels
  float* xmax_out;
  const int* slot_group;
  // FP8 tier (fp8 = 1): X and C are E4M3 copies, rows of ld bytes (launch_assign_bf16's ldxb /
  // ldcb count bytes); key = acc * (xscale[row] * *cscale) + cinit[j]; xscale is indexed like
  // thr_in in the candidate pass (row0 + row) and like xnorm otherwise (out0 + row)
  int fp8;
  const float* xscale;
  const float* cscale;
  // test hook of the FP32 tier (kmgb_debug_withhold_stage): the producer issues no TMA load for
  // pipeline steps >= test_withhold (0: every step), and every wait gives up after
  // test_wait_cycles SM cycles (0: KMGB_WAIT_CYCLES)
  long long test_withhold;
  unsigned long long test_wait_cycles;
};

// Many problems of one dimension in one launch (batched Lloyd): problem p owns rows
// R_p .. row_end[p]-1 of X (R_p a multiple of 128) and centers c_off[p] .. c_off[p]+k[p]-1.
struct GroupArgs {
  const int* tile_prob;       // [tiles] problem of each 128-row tile
  const int* c_off;           // [P] first center of the problem (global index)
  const int* k;               // [P] centers of the problem
  const long long* row_end;   // [P] one past the problem's last row
  const int* done;            // [P] nullable: problems whose loop has stopped (skipped)
};

// FP32 SIMT assignment. X: [n][ldx] FP32, Cop: [k][ldc] FP32 (ld multiples of 4 floats).
// With grp: `tiles` 128-row tiles of grouped problems (a.n = rows of X, a.k = all centers);
// labels are global center indices.
cudaError_t launch_assign_fp32(const float* X, long long ldx, const float* Cop, long long ldc,
                               const AssignArgs& a, cudaStream_t s,
                               const GroupArgs* grp = nullptr, long long tiles = 0);
float assign_fp32_gamma(int d);

// tcgen05 BF16 assignment. Xb: [n][ldb] BF16, Cb: [k][ldb] BF16, ldb a multiple of 8. With the
// residual planes Xl / Cl (x - bf16(x), same layout; both nullable) the split tier computes
// x_hi.c_hi + x_hi.c_lo + x_lo.c_hi; with Cl but no Xl (every x a BF16 number) it computes
// x.c_hi + x.c_lo, two products with the bound of an exact x.
cudaError_t launch_assign_bf16(const void* Xb, const void* Xl, long long ldxb, const void* Cb,
                               const void* Cl, long long ldcb, const AssignArgs& a,
                               cudaStream_t s);
float assign_bf16_gamma(int d);
// D up to 512 with one BF16 plane of the points (plain tier, split tier with BF16-valued points,
// store mode), up to 320 with two (split tier): the unit's points stay in shared memory.
bool bf16_tc_supported(int d, int planes = 1);
// The FP8 tier (AssignArgs.fp8 through launch_assign_bf16): D up to 512.
bool fp8_tc_supported(int d);

// Exact re-rank of flagged points. mode 0 (Lloyd): FP64 arg-min of sum_d (x_d - c_d)^2.
// mode 1 (expansion, caller norms): FP64 arg-min of nb_j - 2 x.c_j with the given nb.
struct RerankArgs {
  const float* X; long long ldx;
  const float* C; long long ldc;   // usable-center operand copy (zero rows for NaN centers)
  const float* cn;                 // [k] +inf marks an unusable center (mode 0)
  const float* nb;                 // [k] caller norms (mode 1)
  const float* xnorm;              // [n] (mode 1 bound)
  const float* cmax;               // (mode 1 bound)
  const int* list; const int* count;
  int* labels;
  unsigned long long* stats;       // [2]: points re-ranked, points that needed FP64
  long long n; int k; int d;
  int mode;
  long long max_list;
  const int* stop;
};
cudaError_t launch_rerank(const RerankArgs& a, cudaStream_t s);
// FP32 stage of the Lloyd re-rank (mode 0): certifies what FP32 can, passes the rest to list2.
// hi2[slot] receives the FP32 upper end of the best center of every point passed on.
cudaError_t launch_rerank_tiled(const RerankArgs& a, int* list2, int* count2, float* hi2,
                                cudaStream_t s);
// Grouped problems (batched Lloyd): one CTA per flagged row over its own problem's centers
// (FP32 band, then FP64); a.C / a.cn cover all problems' centers, a.stats (nullable) counts.
// With cand (capacity cand_cap list slots of kMaxCand): flagged rows in slots below cand_cap only
// record their FP32 band as candidates (cand_cnt -1 past kMaxCand) for launch_resolve_candidates;
// the others, and every row without cand, are settled here (FP32 band, then FP64).
cudaError_t launch_rerank_grouped(const RerankArgs& a, const GroupArgs& g, cudaStream_t s,
                                  int* cand = nullptr, int* cand_cnt = nullptr,
                                  long long cand_cap = 0);
// FP64 stage over list2 (one CTA per point), candidates bounded by hi2.
cudaError_t launch_rerank_exact(const RerankArgs& a, const float* hi2, cudaStream_t s);
// Candidate re-rank of the BF16 tiers: compact copy of up to `cap` flagged rows (the rest go to
// `over`), then FP64 resolution of their recorded candidates (overflowing points are appended
// to `over`). With row_map (the router's routed scan), list entries are routed rows whose
// candidates are stored per routed row and whose FP32 row is X[row_map[entry]].
// row_bytes: bytes per row of Xb / Xl (a multiple of 16); xs / xsC (nullable): per-row scales
// of the FP8 tier copied along.
cudaError_t launch_gather_flagged(const int* list, const int* count, long long cap,
                                  const void* Xb, const void* Xl, long long row_bytes,
                                  const float* thr, void* XbC, void* XlC, float* thrC, int* over,
                                  int* over_count, const int* stop, cudaStream_t s,
                                  const float* xs = nullptr, float* xsC = nullptr);
cudaError_t launch_resolve_candidates(const int* list, const int* count, long long max_list,
                                      const int* cand, const int* cand_cnt, const float* X,
                                      long long ldx, const float* C, long long ldc, const float* cn,
                                      int d, int* labels, int* over, int* over_count,
                                      const int* stop, cudaStream_t s,
                                      const int* row_map = nullptr);
// stats[0] += counts[0] (points flagged by the assignment), stats[1] += counts[full_idx]
// (points that needed a full rescan of the centers).
// Audit of certified labels (rerank.cu): `rows` sampled rows (at most kAuditMaxRows) against
// the FP64 arg-min over all k centers; ws holds 4 + 2 * kAuditMaxRows words, zero before the
// first audit ([0] rows audited, [1] violations, [3] 1 + the last violating row).
constexpr int kAuditMaxRows = 256;
// With grp (batched problems): each sampled row against its own problem's centers; padding rows
// and rows of stopped problems are skipped (not counted in ws[0]).
cudaError_t launch_audit_labels(const float* X, long long ldx, long long n, int d, const float* C,
                                long long ldc, int k, const int* labels, unsigned long long* ws,
                                int rows, const int* stop, cudaStream_t s,
                                const GroupArgs* grp = nullptr);
cudaError_t launch_count_stats(const int* counts, int full_idx, unsigned long long* stats,
                               const int* stop, cudaStream_t s);

// Center preparation: from the official centers C[k][ldc] write the operand copy Cop (NaN
// rows -> 0), optional BF16 copy Cb[k][ldcb], cn (+inf for NaN rows) and atomically raise
// *cmax (must be zeroed before).
// cinit (nullable, round_up(k,128) floats) receives -cn/2 per usable center and -3e38 for
// unusable centers and padding; cbias (nullable, round_up(k,128) rows of kBiasCols BF16) the same
// start values split exactly into three BF16 numbers (columns 0..2, the rest zero), the B
// operand of the pair kernel's start-value MMA.
constexpr int kBiasCols = 16;
cudaError_t launch_prep_centers(const float* C, long long ldc, int k, int d, float* Cop,
                                void* Cb, long long ldcb, float* cn, float* cmax, cudaStream_t s,
                                const int* stop = nullptr, float* cinit = nullptr,
                                void* Cl = nullptr, void* cbias = nullptr);

// Per-point norms, computed once per data set: qn = ||x||^2 (FP64), xn = upper bound ||x||.
cudaError_t launch_point_norms(const float* X, long long ldx, long long n, int d, double* qn,
                               float* xn, cudaStream_t s);
// FP8 E4M3 copies (the FP8 tier): every row of X scaled by its own power of two sx[row], the
// centers (from the operand copy) by one power of two *cscale derived from *cmax; rows zero
// padded to ld8 bytes (a multiple of 16).
cudaError_t launch_to_fp8(const float* X, long long ldx, long long n, int d, void* X8,
                          long long ld8, float* sx, cudaStream_t s, const int* stop = nullptr);
cudaError_t launch_centers_fp8(const float* Cop, long long ldc, int k, int d, const float* cmax,
                               void* C8, long long ld8, float* cscale, cudaStream_t s,
                               const int* stop = nullptr);
// BF16 copy of the data set (zero padded to ldb columns).
// Xl (nullable) receives the residual plane bf16(x - bf16(x)); inexact (nullable, zeroed by the
// caller) is set to 1 when some value is not a BF16 number.
cudaError_t launch_to_bf16(const float* X, long long ldx, long long n, int d, void* Xb,
                           long long ldb, cudaStream_t s, const int* stop = nullptr,
                           void* Xl = nullptr, int* inexact = nullptr);

// Deterministic update: stable counting sort by label, FP64 piece sums, finalize.
struct UpdateWork {
  // sizes
  long long n; int k; int d; long long ldx; int tile_pts; int ntiles;
  long long max_pieces;
  // buffers (device)
  int* hist;            // [k * ntiles]
  int* scan_tmp;        // [scan_blocks]
  int* label_off;       // [k + 1]
  int* piece_cnt;       // [k + 1] -> exclusive scan = piece start
  int* sorted;          // [n]
  double* part;         // [max_pieces * d]
  double* partq;        // [max_pieces]
  double* sse_k;        // [k][ceil(d/32)] SSE terms per (center, group of 32 dimensions)
  long long* counts;    // [k]
  int* err;
  // stop rule (kmeans.cpp:1194-1237), evaluated on the device by the SSE reduction
  int* stop;            // nullable
  double criterion;
  double* sse_prev;     // previous SSE (0 before the first iteration)
  double* rel_out;      // last relErr
  int* iters_done;      // iterations completed
  int sse_indexed;      // 1: the SSE lands in sse_out[*iters_done] (a run's iteration index,
                        // so one captured iteration serves every iteration of the run)
};
size_t update_scan_tmp_elems(long long elems);
cudaError_t launch_update(const float* X, const double* qn, const int* labels, float* C,
                          long long ldc, int empty_policy, const UpdateWork& w, double* sse_out,
                          cudaStream_t s);

// Per-kernel ABI accumulation across tiles: adds the tile's canonical FP64 per-center sums to
// acc[k][d] and its member counts to acc_counts[k]; finalize writes acc/count (NaN if empty).
template <typename T>
cudaError_t launch_tile_accumulate(const T* X, long long ldx, const int* labels, const UpdateWork& w,
                                   double* acc, int* acc_counts, cudaStream_t s);
template <typename T>
cudaError_t launch_finalize_acc(const double* acc, const int* acc_counts, int k, int d, T* centers,
                                int* counts, cudaStream_t s);
void plan_update_tiles(long long n, int k, int* tile_pts, int* ntiles);
// Host-streamed tiles: per tile, label sort + canonical piece sums (with sum of ||x||^2) added to
// FP64 accumulators accS[k][d], accN[k], accQ[k]; after the last tile, centers, SSE and the stop
// rule from the accumulators.
cudaError_t launch_stream_accumulate(const float* X, long long ldx, const double* qn,
                                     const int* labels, const UpdateWork& w, double* accS,
                                     int* accN, double* accQ, cudaStream_t s);
cudaError_t launch_stream_finalize(const double* accS, const int* accN, const double* accQ,
                                   float* C, long long ldc, int empty_policy, const UpdateWork& w,
                                   double* sse_out, cudaStream_t s);

// Batched Lloyd update (problems of one dimension sharing X and one center matrix; labels are
// global center indices). Device arrays; see launch_update_batched.
struct BatchUpdate {
  int P;                        // problems
  int K;                        // centers of all problems
  long long n_valid;            // rows of all problems (padding rows excluded)
  const long long* row_beg;     // [P] first row of the problem
  const long long* row_end;     // [P] one past its last row
  const int* c_off;             // [P] first center
  const int* k;                 // [P] centers
  const long long* hoff;        // [P] first counter of the problem in hist
  const int* ntiles;            // [P] sort tiles of the problem
  const int* cprob;             // [K] problem of each center
  long long stiles;             // sort tiles of all problems
  const int* stile_prob;        // [stiles]
  const int* stile_local;       // [stiles] tile index inside its problem
  int tile_pts;                 // rows per sort tile
  int kmax;                     // largest k of the problems
  long long hist_elems;         // sum over problems of k * ntiles
  // per-problem loop state (device)
  int* done;                    // [P] 1 once the problem's stop rule fired
  double* sse_prev;             // [P]
  double* rel;                  // [P] last relErr
  int* iters;                   // [P] iterations recorded
  double* sse_hist;             // [P][max_iters]
  int max_iters;
  double criterion;
};
cudaError_t launch_update_batched(const float* X, long long ldx, int d, const double* qn,
                                  const int* labels, float* C, long long ldc, int empty_policy,
                                  const UpdateWork& w, const BatchUpdate& b,
                                  cudaStream_t s);

// Mini-batch gather: rows perm[(start + r) mod m] of Xsrc into Xdst (m_mb rows).
cudaError_t launch_gather_rows(const float* Xsrc, long long ldx, const int* perm, long long m,
                               long long start, long long m_mb, int d, float* Xdst,
                               long long ldd, cudaStream_t s, const int* stop = nullptr);
cudaError_t launch_gather_vec(const double* qsrc, const float* xsrc, const int* perm,
                              long long m, long long start, long long m_mb, double* qdst,
                              float* xdst, cudaStream_t s, const int* stop = nullptr);

// k-means++ (D^2-weighted draws, seeded): k centers from X (n x d, row stride ldx) into C (k x d,
// row stride ldc); picks[k] receives the chosen rows. Work space: d2[kmeanspp_d2_elems(n)],
// blocksum[kmeanspp_blocks(n)], scalars[3]; err: device error word (a bounded wait that gave up).
long long kmeanspp_blocks(long long n);
long long kmeanspp_d2_elems(long long n);
cudaError_t launch_kmeanspp(const float* X, long long ldx, long long n, int d, int k,
                            unsigned long long seed, float* C, long long ldc, int* picks,
                            float* d2, unsigned long long* blocksum, unsigned long long* scalars,
                            int* err, cudaStream_t s);
cudaError_t launch_kmeanspp(const double* X, long long ldx, long long n, int d, int k,
                            unsigned long long seed, double* C, long long ldc, int* picks,
                            double* d2, unsigned long long* blocksum, unsigned long long* scalars,
                            int* err, cudaStream_t s);

constexpr int kSumPiece = 128;
constexpr int kMaxCand = 32;  // candidate centers recorded per flagged point
// BF16 tiers: centers per tensor-core chunk; the start values and diagnostic accumulators are
// padded to a whole number of chunks
constexpr int kCenterPad = 256;

// Host: the reference's shuffle permutation (perm[i] = source row of shuffled row i) and its
// initial picks (srand(42) / rand() % m, kmeans.cpp:554-557, 876-883); engine.cu.
void reference_perm(int m, std::vector<int>& perm);
bool reference_picks(int m, int k, std::vector<int>& picks);

// Message returned by kmgb_last_error() on the calling thread.
void set_last_error(const char* msg);

// Streaming multiprocessors of the current device (cached per device); sizes grids.
int num_sms();

// Test hooks (devmem.cu; kmgb_debug_fail_nth, kmgb_debug_withhold_stage): inject_fault(kind)
// is true for the one event of that kind that a test asked to fail; the library then returns
// the CUDA error that event would have produced instead of performing it.
constexpr int kFaultAlloc = 1;   // device allocation from the pool
constexpr int kFaultCopy = 2;    // host<->device copy of a data set, centers or results
constexpr int kFaultLaunch = 3;  // launch of a Lloyd-phase kernel
bool inject_fault(int kind);
// FP32-tier assignment launches: withhold the TMA loads of pipeline steps >= *withhold (0: off)
// and bound every wait by *wait_cycles SM cycles (0: the default limit).
void test_wait_hook(long long* withhold, unsigned long long* wait_cycles);

// Device memory from the library's stream-ordered pool of the current device (devmem.cu):
// dev_alloc returns memory usable from every stream; dev_free gives it back in the order of s.
cudaError_t dev_alloc(void** p, size_t bytes, cudaStream_t s);
void dev_free(void* p, cudaStream_t s);
cudaError_t dev_release_cached();

}  // namespace kmgb
