/*
 * kmeans_gb300 -- C-ABI of the GB300 (sm_103a) K-means Lloyd hot path.
 *
 * Drop-in boundary for PaulMullowney/kmeans. Three groups of entry points, all `extern "C"`
 * with plain pointers and sizes:
 *
 *  1. The reference's public driver API (main/cpp/kmeans.hpp:44-132): computeKmeansF,
 *     computeKmeansD, kmeansGetErrorString, with the same signatures, enum values and the same
 *     D x K ("K fastest") layout of `result`.
 *  2. The reference's per-kernel API (main/cuda/KmeansCudaKernels.h:174-474): device-pointer
 *     entry points with the same names, argument meaning and kmeansCudaErrorStatus codes.
 *  3. An extension (kmgb_*) that the reference cannot express: explicit initial centers,
 *     labels and per-iteration SSE out, precision tier selection, a resident handle for
 *     repeated runs, and statistics.
 *
 * Everything runs on the calling thread's current CUDA device.
 */
#ifndef KMEANS_GB300_H_
#define KMEANS_GB300_H_

#include <stdbool.h>
#include <stddef.h>

#if defined(__GNUC__)
#define KMGB_EXPORT __attribute__((visibility("default")))
#else
#define KMGB_EXPORT
#endif

#if defined(__cplusplus)
extern "C" {
#endif

/* ---------------------------------------------------------------------------------------
 * 1. Reference driver API
 * ------------------------------------------------------------------------------------- */

/* Same names and values as the reference (main/cpp/kmeans.hpp:44-59). */
typedef enum kmeansErrorStatus {
  KMEANS_SUCCESS = 0,
  KMEANS_ERROR_BUILDDATA = 1,
  KMEANS_ERROR_INITIALIZE = 2,
  KMEANS_ERROR_CLOSEST_CENTERS = 3,
  KMEANS_ERROR_CLUSTER_CENTERS = 4,
  KMEANS_ERROR_COMPACTNESS = 5,
  KMEANS_ERROR_TRANSPOSE = 6,
  KMEANS_ERROR_RESET = 7,
  KMEANS_ERROR_COMPUTE = 8,
  KMEANS_ERROR_GET_CENTERS = 9,
  KMEANS_ERROR_TILING = 10,
  KMEANS_ERROR_COPY_TILE = 11,
  KMEANS_ERROR_CONSTRUCT_MINIBATCH = 12,
  KMEANS_NONCONVERGENCE = 13
} kmeansErrorStatus;

/* Replaces kmeansGetErrorString (main/cpp/kmeans.hpp:66-82); same strings. */
KMGB_EXPORT const char* kmeansGetErrorString(kmeansErrorStatus err);

/* Replaces computeKmeansF (main/cpp/kmeans.hpp:102-107, main/cpp/kmeans.cpp:1316-1361).
 * data: host, m x n row-major. result: host, n x k with result[j*k + i] = dim j of center i;
 * it receives the initial centers, then the final centers. The data are shuffled with
 * std::shuffle(default_random_engine(0)) and the initial centers picked with srand(42)/rand()
 * exactly as the reference does when initAlgorithm is 0 (numRetries is then ignored, as in the
 * reference). initAlgorithm 1 (an extension) draws k-means++ centers with seeds 0 ..
 * numRetries-1 and keeps the run with the lowest final SSE; result then receives that run's
 * initial centers before its final ones. doFullSGEMM (0/1/2) and matrixFormat (0/1) are accepted and
 * all map to the same fused assignment: the split BF16 tensor-core tier when n <= 320, the FP32
 * tier above (the labels are the certified FP64 arg-min in both; the environment variable
 * KMGB_ASSIGN=fp32|bf16|bf16x3 picks a tier). miniBatchFraction < 1 selects the reference's
 * sliding mini-batch windows. Returns KMEANS_NONCONVERGENCE (13) when the relative SSE change
 * is still above `criterion` after maxIters iterations (criterion < 0 always runs maxIters). */
KMGB_EXPORT kmeansErrorStatus computeKmeansF(const float* data, const int m, const int n, const int k,
                                 const float criterion, const int maxIters,
                                 const int numRetries, const int initAlgorithm,
                                 const int doFullSGEMM, const int matrixFormat, float* result,
#if defined(__cplusplus)
                                 const float miniBatchFraction = 1.0f); /* as kmeans.hpp:107 */
#else
                                 const float miniBatchFraction);
#endif

/* Replaces computeKmeansD (main/cpp/kmeans.hpp:127-132, main/cpp/kmeans.cpp:1364-1409), with
 * computeKmeansF's arguments and layouts on FP64 data. Labels are the FP64 arg-min of the
 * direct distance (lowest index on ties); centers are canonical FP64 sums over the counts. Full
 * batches with n <= 320 assign on the tensor cores (the split BF16 tier on FP32 roundings of the
 * data and centers, its bound widened by that rounding, the uncertified points rescanned in
 * FP64); mini-batch windows, wider data and KMGB_ASSIGN=fp32 use the FP64 scan for every point. */
KMGB_EXPORT kmeansErrorStatus computeKmeansD(const double* data, const int m, const int n, const int k,
                                 const double criterion, const int maxIters,
                                 const int numRetries, const int initAlgorithm,
                                 const int doFullSGEMM, const int matrixFormat, double* result,
#if defined(__cplusplus)
                                 const double miniBatchFraction = 1.0); /* as kmeans.hpp:132 */
#else
                                 const double miniBatchFraction);
#endif

/* ---------------------------------------------------------------------------------------
 * 2. Reference per-kernel API (device pointers, asynchronous on the default stream)
 * ------------------------------------------------------------------------------------- */

/* Same names and values as main/cuda/KmeansCudaKernels.h:174-183. */
typedef enum kmeansCudaErrorStatus {
  NO_ERROR = 0,
  ERROR_MATMATMULT = 1,
  ERROR_ROWTRANSFORMMINIMUM = 2,
  ERROR_CLOSESTCENTERS = 3,
  ERROR_CLUSTERCENTERS = 4,
  ERROR_COMPACTNESS = 5,
  ERROR_ROWNORMALIZE = 6,
  ERROR_COLNORMALIZE = 7
} kmeansCudaErrorStatus;

/* Replace MatMatMultF/D (KmeansCudaKernels.h:198-215, MatMatMult.cu:70-110): C = A B for
 * row-major device matrices A (nRowsA x nColsA), B (nColsA x nColsB), C (nRowsA x nColsB), FP32
 * / FP64 FMA accumulation over the columns of A in ascending order; asynchronous on the legacy
 * default stream; ERROR_MATMATMULT for negative sizes or a failed launch. */
KMGB_EXPORT kmeansCudaErrorStatus MatMatMultF(const int nRowsA, const int nColsA, const float* A,
                                              const int nColsB, const float* B, float* C);
KMGB_EXPORT kmeansCudaErrorStatus MatMatMultD(const int nRowsA, const int nColsA, const double* A,
                                              const int nColsB, const double* B, double* C);

/* Replaces ClosestCentersF (KmeansCudaKernels.h:238-244, ClosestCenters.cu:392-403).
 * A: nRowsA x nColsA row-major; B: nColsA x nColsB (centers are columns, K fastest);
 * CindicesFinal[m0 + i] = arg-min_j normColsOfB_squared[j] - 2 A_i.B_j, lowest j on ties,
 * equal to the FP64 evaluation of that expression. Bpadded, normRowsOfA_squared, nColsC, C and
 * Cindices are the reference's scratch arguments: accepted, not required (may be NULL). */
KMGB_EXPORT kmeansCudaErrorStatus ClosestCentersF(const int m0, const int nRowsA, const int nColsA,
                                      const float* A, const int nColsB, const float* B,
                                      float* Bpadded, const float* normRowsOfA_squared,
                                      const float* normColsOfB_squared, const int nColsC,
                                      float* C, int* Cindices, int* CindicesFinal);
/* Replaces ClosestCentersD (KmeansCudaKernels.h:267-273): FP64 data, exact FP64 arg-min. */
KMGB_EXPORT kmeansCudaErrorStatus ClosestCentersD(const int m0, const int nRowsA, const int nColsA,
                                      const double* A, const int nColsB, const double* B,
                                      double* Bpadded, const double* normRowsOfA_squared,
                                      const double* normColsOfB_squared, const int nColsC,
                                      double* C, int* Cindices, int* CindicesFinal);

/* Replace rowTransformMinimumF/D (KmeansCudaKernels.h:290-313, RowTransformMinimum.cu:3-99):
 * output[m0+i] = arg-min_j normA[i] + normB[j] - 2 input[i*n+j], evaluated with the reference's
 * expression and rounding, lowest j on ties. normA is indexed from the start of the tile as in
 * the reference (RowTransformMinimum.cu:21). */
KMGB_EXPORT kmeansCudaErrorStatus rowTransformMinimumF(const int m0, const int m, const int n,
                                           const float* normRowsOfA_squared,
                                           const float* normColsOfB_squared, const float* input,
                                           int* output);
KMGB_EXPORT kmeansCudaErrorStatus rowTransformMinimumD(const int m0, const int m, const int n,
                                           const double* normRowsOfA_squared,
                                           const double* normColsOfB_squared,
                                           const double* input, int* output);

/* Replace ClusterCentersF/D (KmeansCudaKernels.h:337-369, ClusterCenters.cu:101-188):
 * data: m x n rows of the tile, indices[m0 + i] their labels. Sums accumulate across calls
 * in counts_large/centers_large (K ints / K x n FP64 values viewed through the caller's
 * buffers, which must hold at least K x n doubles and K ints); on lastTile the means are written
 * to centers (K x n row-major, NaN for an empty cluster) and the member counts to counts. */
KMGB_EXPORT kmeansCudaErrorStatus ClusterCentersF(const int m0, const int m, const int n, const int k,
                                      const bool lastTile, const float* data, const int* indices,
                                      float* centers_large, int* counts_large, float* centers,
                                      int* counts);
KMGB_EXPORT kmeansCudaErrorStatus ClusterCentersD(const int m0, const int m, const int n, const int k,
                                      const bool lastTile, const double* data, const int* indices,
                                      double* centers_large, int* counts_large, double* centers,
                                      int* counts);

/* No counterpart in the reference. ClusterCentersF for callers that cannot allocate device
 * memory (programs that reserve all device memory up front and forbid allocation afterwards, or
 * whose memory pool owns the GPU): same arguments and results as ClusterCentersF, but the
 * working memory (label histogram, sorted ids, FP64 piece sums) comes from one 8 MiB array in
 * device global memory that the library holds on every GPU that loads it, instead of the
 * stream-ordered allocator; nothing is allocated. Sizes that need more than 8 MiB of working
 * memory (roughly (m/128 + k) * n * 8 + (m + 2k + k*tiles) * 4 bytes) return
 * ERROR_CLUSTERCENTERS with a message in kmgb_last_error(). The first call on a device looks up
 * the array's device address: make it before any stream capture. All calls share the array and
 * it keeps the last call's contents; calls that overlap on the GPU race and must be serialised
 * by the caller. */
KMGB_EXPORT kmeansCudaErrorStatus ClusterCentersF_noalloc(const int m0, const int m, const int n,
                                                          const int k, const bool lastTile,
                                                          const float* data, const int* indices,
                                                          float* centers_large, int* counts_large,
                                                          float* centers, int* counts);

/* Replace CompactnessF/D (KmeansCudaKernels.h:389-414, Compactness.cu:62-139): the squared
 * distance of every row to centers[indices[m0+i]] (K x n row-major) is added to a running FP64
 * total kept inside the caller's buffer (compactness[2..3] viewed as one double for F,
 * compactness[1] for D; the caller zeroes the buffer before the first tile, as the reference's
 * reset does); on lastTile compactness[0] receives the total. */
KMGB_EXPORT kmeansCudaErrorStatus CompactnessF(const int m0, const int m, const bool lastTile, const int n,
                                   const int k, const float* data, const int* indices,
                                   const float* centers, float* compactness);
KMGB_EXPORT kmeansCudaErrorStatus CompactnessD(const int m0, const int m, const bool lastTile, const int n,
                                   const int k, const double* data, const int* indices,
                                   const double* centers, double* compactness);

/* Replace rowNormalizeF/D and colNormalizeF/D (KmeansCudaKernels.h:428-474,
 * Normalize.cu:3-47): squared L2 norm of each row (output[m0+i]) / of each column of an m x n
 * matrix, accumulated in FP64 and rounded once. */
KMGB_EXPORT kmeansCudaErrorStatus rowNormalizeF(const int m0, const int m, const int n, const float* input,
                                    float* output);
KMGB_EXPORT kmeansCudaErrorStatus rowNormalizeD(const int m0, const int m, const int n, const double* input,
                                    double* output);
KMGB_EXPORT kmeansCudaErrorStatus colNormalizeF(const int m, const int n, const float* input, float* output);
KMGB_EXPORT kmeansCudaErrorStatus colNormalizeD(const int m, const int n, const double* input,
                                    double* output);

/* ---------------------------------------------------------------------------------------
 * 3. Extension (no counterpart in the reference ABI, which returns neither labels nor SSE)
 * ------------------------------------------------------------------------------------- */

enum kmgb_assign_tier {
  KMGB_ASSIGN_FP32 = 0,  /* plain FP32 fused kernel (TMA + FFMA) */
  KMGB_ASSIGN_BF16 = 1,  /* tcgen05 BF16 tensor cores, FP32 accumulate in TMEM (D <= 512) */
  KMGB_ASSIGN_BF16X3 = 2, /* tcgen05 split BF16: x.c = xh.ch + xh.cl + xl.ch (D <= 320) */
  KMGB_ASSIGN_FP8 = 3,    /* tcgen05 FP8 E4M3 (kind::f8f6f4), every point row with its own
                             power-of-two scale, the centers with one; full batches of resident
                             data, D <= 512; labels certified against the E4M3 bound and settled
                             exactly like the BF16 tiers' */
  KMGB_ASSIGN_AUTO = 4    /* kmgb_lloyd_batched_f32 only: every dimension's problems take the
                             tier (FP32 or BF16X3) with the smaller time predicted from a measured
                             cost table (kmeans_gb300/autotune.py) by (d, k) bucket and rows */
};

enum kmgb_empty_policy {
  KMGB_EMPTY_NAN = 0, /* reference behaviour: 0/0 = NaN center (ClusterCenters.cu:81) */
  KMGB_EMPTY_KEEP = 1 /* keep the previous center */
};

/* Initialisation when no initial centers are given. initAlgorithm of computeKmeansF/D takes the
 * same values. */
enum kmgb_init_algorithm {
  KMGB_INIT_REFERENCE = 0, /* the reference's shuffle + srand(42) picks (kmeans.cpp:554-557, 876-888) */
  KMGB_INIT_KMEANSPP = 1   /* k-means++: D^2-weighted seeded draws, see kmgb_kmeanspp_f32 */
};

typedef struct kmgb_options {
  int assign_tier;           /* kmgb_assign_tier */
  int certify;               /* 1: labels equal the FP64 arg-min (margin test + re-rank) */
  int empty_policy;          /* kmgb_empty_policy */
  int max_iters;             /* iterations (upper bound when criterion >= 0) */
  double criterion;          /* stop when |dSSE|/SSE <= criterion; < 0: run max_iters */
  float mini_batch_fraction; /* < 1: reference mini-batch windows of (int)(f*m) rows */
  int stream_tile_rows;      /* > 0 and < n: host-streamed tiles (the reference's out-of-memory
                                path): X stays in host memory and passes through two device
                                tile buffers of this many rows every iteration; the host array
                                must stay valid while the handle runs. 0: X resident in HBM */
  int init_algorithm;        /* initial centers when none are given: kmgb_init_algorithm */
  int num_retries;           /* k-means++: runs seeded seed, seed+1, ...; the run with the lowest
                                final SSE is returned (< 1 counts as 1) */
  unsigned long long seed;   /* k-means++ seed */
  int router;                /* 1: learned router (needs a BF16 tier, full batches, resident
                                data): after the first iteration an MLP routes every point to one
                                group of centers, the point is scanned against that group only and
                                certified (see kmgb_get_router_stats); uncertified points take the
                                full scan, so labels are unchanged */
  int router_groups;         /* G, groups of centers (0: 256) */
  int router_retrain;        /* retrain every this many iterations (0: 5) */
  int router_hidden;         /* hidden units of the MLP, 256 or 512 (0: 512) */
} kmgb_options;

typedef struct kmgb_stats {
  int iterations;
  int status;                      /* kmeansErrorStatus of the run */
  unsigned long long reranked;     /* points whose approximate margin did not certify the label
                                      (all iterations); each is settled exactly */
  unsigned long long reranked_fp64;/* of those, points that needed a full rescan of the centers
                                      (FP32 then FP64) instead of their recorded candidates */
  long long empty_clusters;        /* empty clusters seen after the last update */
  double ms_total;                 /* wall time of the iterations (CUDA events) */
  long long reserved[8];           /* with the router: [0] points routed to a group scan, [1]
                                      of those certified, [2] points that took the full scan,
                                      [3] trainings, [4] training wall time (us), [5] routed
                                      points whose in-group margin took the candidate pass;
                                      certified resident runs: [6] rows audited, [7] audit
                                      violations -- every iteration a sample of rows (64 by
                                      default, KMGB_AUDIT_ROWS, fewer when k x d is large) is
                                      checked against the FP64 arg-min over all centers, so a
                                      failure of a rounding model behind the certificate shows
                                      as a violation count instead of a silently wrong label */
} kmgb_stats;

/* The learned router's record (kmgb_get_router_stats); counters sum over the iterations run. */
typedef struct kmgb_router_stats {
  long long trainings;        /* trainings run (the groups are formed at the first) */
  double train_ms;            /* wall time of the trainings, grouping included */
  double group_ms;            /* of which forming the groups of centers */
  double last_loss;           /* mean cross-entropy of the last training batch */
  double last_accuracy;       /* share of that batch routed to its label's group */
  int groups_nonempty;        /* groups holding at least one center */
  int components;             /* components of linked centers packed into the groups */
  int max_group;              /* centers of the largest group */
  int max_component;          /* centers of the largest component */
  unsigned long long scan_chunks; /* sum over routed points of their group's 256-center chunks
                                     (a full scan is ceil(k / 256) per point) */
  unsigned long long routed;  /* points routed to a group scan */
  unsigned long long flagged; /* of those, points whose in-group margin took the candidate pass */
  unsigned long long certified; /* points whose group winner was certified as the arg-min */
  unsigned long long fallback;  /* points that took the full scan instead */
  long long routed_iterations;  /* iterations that ran the routed scan */
  long long device_bytes;       /* device memory of the router (fallback buffers excluded) */
  double stage_ms[7];           /* with profiling on (kmgb_set_profiling): CUDA-event ms of the
                                   routed assignment's stages summed over the routed iterations:
                                   centers in group order, center separation, network inference,
                                   sort by group, group scan, in-group near ties, certificate */
  long long reserved[4];
} kmgb_router_stats;

/* The reference's initial centers, computed on the host: k x d row-major copies of data rows
 * perm[picks[i]], perm from std::shuffle(default_random_engine(0)) and picks from srand(42) /
 * rand() % m with the unsorted binary_search (main/cpp/kmeans.cpp:554-557, 876-888). perm and
 * picks (each nullable) receive the permutation (m) and the picks (k). Needs no GPU. */
KMGB_EXPORT int kmgb_reference_init(const float* data, int m, int d, int k, float* centers,
                                    int* perm, int* picks);

/* k-means++ initial centers (Arthur & Vassilvitskii, 2007), reproducible bit for bit for a seed:
 * draw 0 is uniform; draw r picks a point with probability proportional to its weight
 * q = trunc(D^2 * 2^31 / max D^2), D^2 = squared distance (in the data's precision) to the
 * nearest center drawn so far, from the 53-bit number u = splitmix64(splitmix64(seed) + r) >> 11
 * as the point whose interval of the running sum of q holds (u * sum q) >> 53.
 * X: n x d row-major (host or device); centers: k x d row-major (host or device, nullable);
 * picks: the k chosen rows (host, nullable). Runs on the GPU; the data set must fit in HBM. */
KMGB_EXPORT int kmgb_kmeanspp_f32(const float* X, long long n, int d, int k, unsigned long long seed,
                                  float* centers, int* picks);
KMGB_EXPORT int kmgb_kmeanspp_f64(const double* X, long long n, int d, int k,
                                  unsigned long long seed, double* centers, int* picks);

/* Defaults: FP32 tier, certify on, NaN policy, 20 iterations, criterion -1, full batch,
 * reference initialisation, one retry, seed 0. */
KMGB_EXPORT void kmgb_default_options(kmgb_options* opt);

/* One-shot Lloyd run. X: n x d row-major FP32 (host or device pointer). init: k x d row-major
 * initial centers (host or device), or NULL for opt->init_algorithm (with opt->num_retries runs
 * for k-means++, keeping the lowest final SSE). Outputs (host or
 * device, each may be NULL): centers k x d row-major, labels[n] of the last assignment
 * (source-row order; -1 outside the last mini-batch window), sse[max_iters] per iteration
 * (FP64, against the updated centers, as the reference's compactness). */
KMGB_EXPORT int kmgb_lloyd_f32(const float* X, long long n, int d, int k, const float* init,
                   const kmgb_options* opt, float* centers, int* labels, double* sse,
                   kmgb_stats* stats);

/* Batched Lloyd: many independent problems in one call (e.g. 10,000 problems of 256..200,000
 * points, D 16..128, K up to a few hundred). Problems of the same dimension share device
 * buffers and every phase of an iteration is one launch over all of them; each problem follows
 * exactly the single-problem semantics (kmgb_lloyd_f32 with the FP32 tier: FP64 arg-min labels,
 * canonical FP64 center sums, FP64 SSE, its own stop rule). */
typedef struct kmgb_problem {
  const float* X;     /* n x d row-major FP32 (host or device) */
  long long n;
  int d;
  int k;
  const float* init;  /* k x d initial centers (host or device), or NULL: the reference
                         initialisation of this problem (needs k <= n) */
  float* centers;     /* out, host, nullable: k x d final centers */
  int* labels;        /* out, host, nullable: n labels of the last assignment */
  double* sse;        /* out, host, nullable: SSE per iteration (opt->max_iters entries) */
  int iterations;     /* out: iterations run */
  int status;         /* out: KMEANS_SUCCESS or KMEANS_NONCONVERGENCE */
  long long reserved[4];
} kmgb_problem;

/* opt: max_iters, criterion, empty_policy, certify and assign_tier (FP32, BF16, BF16X3 or AUTO:
 * per dimension from the tuned cost table) are used; mini_batch_fraction 1, stream_tile_rows 0,
 * init_algorithm KMGB_INIT_REFERENCE. Problems of one dimension and tier form a group whose
 * iteration is captured once as a CUDA graph and replayed (KMGB_GRAPHS=0: kernel by kernel).
 * stats (nullable): iterations = the largest over the problems, reranked = rows settled by the
 * exact re-rank, ms_total = GPU time of the iterations (CUDA events, summed over the groups),
 * reserved[0] = wall time of the whole call in microseconds (uploads, initialisation and result
 * copies included), reserved[1..4] = microseconds of center preparation, assignment, re-rank and
 * update summed over the iterations (CUDA events; kernel-by-kernel runs only), reserved[5] =
 * iteration-graph launches, reserved[6] = groups, reserved[7] = the label audit of certified
 * runs: rows audited (bits 24 and up) and violations found (bits 0-23, saturating) -- every
 * iteration of every group KMGB_AUDIT_ROWS sampled rows (default 64) are checked against the
 * FP64 arg-min over their own problem's centers (padding rows and stopped problems skipped). */
KMGB_EXPORT int kmgb_lloyd_batched_f32(kmgb_problem* problems, int count, const kmgb_options* opt,
                                       kmgb_stats* stats);

/* Resident handle: data uploaded once, iterations run on the handle's own stream. */
typedef struct kmgb_handle kmgb_handle;
KMGB_EXPORT int kmgb_create(kmgb_handle** h, long long n, int d, int k, const kmgb_options* opt);
/* kmgb_set_data copies the n x d rows of X (host or device memory) into the handle; a host
 * buffer may be reused as soon as it returns, a device buffer once the handle's stream has
 * passed the copy (kmgb_synchronize). */
KMGB_EXPORT int kmgb_set_data(kmgb_handle* h, const float* X, int x_on_device);
KMGB_EXPORT int kmgb_set_centers(kmgb_handle* h, const float* C, int c_on_device); /* NULL: reference init */
/* k-means++ centers from the resident data (not for host-streamed handles); picks: k rows (host,
 * nullable). Resets the mini-batch window to the first one. */
KMGB_EXPORT int kmgb_init_kmeanspp(kmgb_handle* h, unsigned long long seed, int* picks);
/* Runs up to `iters` iterations from the current centers (asynchronous when criterion < 0). */
KMGB_EXPORT int kmgb_run(kmgb_handle* h, int iters, double criterion);
KMGB_EXPORT int kmgb_synchronize(kmgb_handle* h);
KMGB_EXPORT int kmgb_get_centers(kmgb_handle* h, float* C, int c_on_device);
KMGB_EXPORT int kmgb_get_labels(kmgb_handle* h, int* labels, int on_device);
KMGB_EXPORT int kmgb_get_sse(kmgb_handle* h, double* sse, int max_count); /* returns the count written */
KMGB_EXPORT int kmgb_get_stats(kmgb_handle* h, kmgb_stats* stats);
/* The router's record (all zero when the handle runs without it). No reference counterpart:
 * the reference scans every center for every point (ClosestCenters.cu:46-83). */
KMGB_EXPORT int kmgb_get_router_stats(kmgb_handle* h, kmgb_router_stats* stats);
/* The router's network alone, for checking it: trains the MLP X (rows x d, host) -> groups with
 * labels y (host, in [0, groups)) from the flat parameters `params` (host, in/out: W1 hidden x d,
 * b1, W2 groups x hidden, b2, row-major) with Adam (lr, betas 0.9 / 0.999, eps 1e-8) on
 * consecutive batches of `batch` rows, `steps` steps. steps == 0: one forward and backward pass
 * over the first batch, its gradients in grads_out (host, nullable) and the parameters unchanged.
 * loss (nullable): the mean cross-entropy of the last batch before its update. */
KMGB_EXPORT int kmgb_router_mlp_train(const float* X, int rows, int d, const int* y, int hidden,
                                      int groups, float* params, int batch, int steps, float lr,
                                      double* loss, float* grads_out);
KMGB_EXPORT void* kmgb_stream(kmgb_handle* h); /* cudaStream_t of the handle */
KMGB_EXPORT int kmgb_destroy(kmgb_handle* h);

/* Sharded Lloyd (points partitioned by rows over ranks or GPUs; no reference counterpart: the
 * reference runs on one GPU, and its update and compactness, kmeans.cpp:1018-1104, are what the
 * ranks exchange). Each rank holds its rows in a full-batch handle with the same centers.
 * kmgb_shard_partials assigns the handle's rows to its current centers (labels as kmgb_run's:
 * the FP64 arg-min) and writes the canonical FP64 sums of those rows per cluster: S (k x d,
 * row-major), counts (k), Q (k, sums of ||x||^2). The caller adds every rank's S, counts and Q
 * in rank order (0 + S_0 + S_1 + ..., in FP64) and gives the totals to kmgb_shard_update on every
 * rank: the new centers (the handle's, with its empty-cluster policy) and the iteration's SSE
 * against them (sse: host). The result equals a single handle whose rows are streamed in tiles
 * equal to the shards (opt.stream_tile_rows). Pointers are host memory (on_device 0) or device
 * memory (on_device 1). */
KMGB_EXPORT int kmgb_shard_partials(kmgb_handle* h, double* S, int* counts, double* Q,
                                    int on_device);
KMGB_EXPORT int kmgb_shard_update(kmgb_handle* h, const double* S, const int* counts,
                                  const double* Q, double* sse, int on_device);

/* Diagnostic: raw tcgen05 accumulators x.c_j - ||c_j||^2/2 for every point and center, as the
 * BF16 (split = 0), split BF16 (split = 1), split BF16 with BF16-valued X (split = 2: the two
 * products x.c_hi + x.c_lo; X must hold BF16 numbers) or FP8 (split = 3: sx sc (x8.c8))
 * assignment kernel computes them. X: n x d, C: k x d,
 * host row-major FP32; out: host n x k. For validating the accumulation-error model on a
 * device; allocates device memory, small problems only. */
KMGB_EXPORT int kmgb_tc_accumulators(const float* X, long long n, int d, const float* C, int k,
                                     int split, float* out);

/* Phase timing: with profiling on, CUDA events on the handle's stream bracket every phase of
 * every iteration. kmgb_get_phase_ms waits for the stream and returns, summed over the
 * iterations run since the previous call, ms[0] center preparation, ms[1] assignment kernel,
 * ms[2] exact re-rank, ms[3] update (sort, sums, SSE); *iters = iterations covered. */
KMGB_EXPORT int kmgb_set_profiling(kmgb_handle* h, int on);
KMGB_EXPORT int kmgb_get_phase_ms(kmgb_handle* h, double* ms, int* iters);
/* Kernels launched by this library since the process started. */
KMGB_EXPORT long long kmgb_launch_count(void);
/* Handles take their device memory from a stream-ordered pool per device that keeps freed
 * memory for the next handle (no reference counterpart: the reference allocates and frees with
 * cudaMalloc/cudaFree in kmeans.cpp:577-683 and its destructor, kmeans.cpp:145-244). This call waits for the current
 * device and returns every pool's unused memory to the device; 0 on success. Setting
 * KMGB_POOL=0 in the environment makes every free return its memory at once. */
KMGB_EXPORT int kmgb_release_cached_memory(void);

/* Test hooks for failure paths (no reference counterpart; the reference reports failures only
 * through its error enums, kmeans.hpp:44-59). kmgb_debug_fail_nth makes the nth later event of a
 * kind fail once, as the CUDA call would have failed: kind 1 = a device allocation from the
 * library's pool, 2 = a host<->device copy of a data set, centers or results, 3 = the launch of a
 * Lloyd-phase kernel (assignment, re-rank, update, center preparation, norms, BF16 conversion);
 * nth <= 0 disarms it. The call that meets the failure returns the kmeansErrorStatus of its phase
 * and releases what it allocated. Process-wide, not thread-safe with concurrent calls. */
KMGB_EXPORT void kmgb_debug_fail_nth(int kind, long long nth);
/* Test hook: FP32-tier assignment launches of handles run after this call issue no TMA load for
 * pipeline step `stage` and later (stage > 0; 0 disarms), and every wait of that kernel gives up
 * after wait_cycles SM cycles (0: the default, about 2 s). The wait for the withheld step runs
 * out, the kernel records KMGB_DEV_TIMEOUT_FULL in the handle's device error word and returns
 * (no copy is left in flight), and the run reports KMEANS_ERROR_CLOSEST_CENTERS. */
KMGB_EXPORT void kmgb_debug_withhold_stage(long long stage, unsigned long long wait_cycles);
/* Bytes of the current device's library pool handed out and not yet given back (-1 on error). */
KMGB_EXPORT long long kmgb_debug_pool_used_bytes(void);
/* Test hook: one audit of `rows` (1..256) sampled rows of device data X (n x d, row stride ldx
 * floats) against the FP64 arg-min over the device centers C (k x d, row stride ldc): a label is
 * a violation when its FP64 distance exceeds the smallest one. out[0] = rows audited, out[1] =
 * violations, out[2] = 1 + the last violating row (0: none). 0 on success. */
KMGB_EXPORT int kmgb_debug_audit(const float* X, long long n, int d, long long ldx, const float* C,
                                 int k, long long ldc, const int* labels, int rows,
                                 unsigned long long* out);

/* Last error message of the calling thread (empty string if none). */
KMGB_EXPORT const char* kmgb_last_error(void);
/* Library constants: piece size of the canonical FP64 center sums, version. */
KMGB_EXPORT int kmgb_sum_piece(void);
KMGB_EXPORT const char* kmgb_version(void);

#if defined(__cplusplus)
}
#endif

#endif /* KMEANS_GB300_H_ */
