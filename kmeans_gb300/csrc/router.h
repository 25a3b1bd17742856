// Internal interface of the learned router (router_mlp.cu: the network; router.cu: groups,
// inference, routed scan and certificate). Not part of the public C-ABI.
#pragma once

#include <cuda_runtime.h>

#include <vector>

namespace kmgb {

enum { kEpiNone = 0, kEpiBias = 1, kEpiBiasRelu = 2, kEpiMask = 3 };

struct MlpShape {
  int d;       // input dimension
  int hidden;  // hidden units
  int groups;  // output classes (groups of centers)
};

struct AdamCfg {
  float lr, beta1, beta2, eps;
};

// Parameters are one flat FP32 vector [W1 (hidden x d) | b1 (hidden) | W2 (groups x hidden) |
// b2 (groups)], row-major; gradients have the same layout.
long long mlp_param_count(const MlpShape& sh);
// Hd = relu(Xs W1^T + b1) (rows x hidden), Z = Hd W2^T + b2 (rows x groups).
cudaError_t mlp_forward(const MlpShape& sh, const float* params, const float* Xs, int rows,
                        float* Hd, float* Z, cudaStream_t s);
// Forward, softmax cross-entropy against y and backward over `rows` rows; the loss and its
// gradient are means over batch_norm_rows. grads: the flat gradient vector; loss_rows[rows].
// part: scratch of mlp_split_scratch(sh) floats for the weight gradients' split over the batch.
cudaError_t mlp_backward(const MlpShape& sh, const float* params, const float* Xs, const int* y,
                         int rows, int batch_norm_rows, float* Hd, float* Z, float* dZ,
                         float* dHd, float* grads, float* loss_rows, cudaStream_t s, float* part,
                         long long part_elems);
long long mlp_split_scratch(const MlpShape& sh);
// One Adam step (step = 1, 2, ...) over n parameters.
cudaError_t mlp_adam(float* params, const float* grads, float* m, float* v, long long n,
                     const AdamCfg& c, long long step, cudaStream_t s);

// What the routed assignment reads and writes of a handle (device pointers).
struct RouterIO {
  long long n;          // rows of the data set
  int d, k;
  long long ldx, ldb;   // FP32 / BF16 row strides
  const float* X;       // n x ldx FP32
  const void* Xb;       // n x ldb BF16 (value plane)
  const void* Xl;       // n x ldb BF16 residual plane, or null (every x a BF16 number / plain tier)
  const float* xn;      // [n] upper bound of ||x||
  const float* C;       // k x ldx official centers (NaN rows: empty clusters)
  const float* Cop;     // k x ldx operand copy (NaN rows zeroed)
  const void* Cb;       // k x ldb BF16 centers
  const void* Cl;       // k x ldb BF16 residual of the centers, or null (plain tier)
  const float* cn;      // [k] fl(||c||^2), +inf for unusable centers
  const float* cinit;   // [round_up(k, 256)] -||c||^2/2, unusable: -3e38
  const void* cbias;    // nullable: the same as BF16 pieces (kBiasCols per center), see
                        // launch_prep_centers
  const float* cmax;    // device scalar: max ||c|| over usable centers
  int* labels;          // [n] out: labels of the certified points
  int* err;             // device error word
  const int* stop;      // device stop flag (nullable)
};

struct Router;
struct RouterStats {
  long long trainings = 0;
  double train_ms = 0.0;       // host wall time of the trainings (grouping included)
  double group_ms = 0.0;       // of which the grouping of the centers
  double last_loss = 0.0;      // mean training loss of the last epoch of the last training
  double last_accuracy = 0.0;  // share of the training sample routed to its label's group
  int groups_nonempty = 0;
  int components = 0;
  int max_group = 0;       // centers of the largest group
  int max_component = 0;   // centers of the largest component
  unsigned long long scan_chunks = 0;  // sum over routed points of their group's 256-center chunks
  // device-side counters summed over routed iterations: points routed to a group scan, points
  // whose in-group margin needed the candidate pass, points certified by the group rule, points
  // sent to the full scan
  unsigned long long routed = 0, flagged = 0, certified = 0, fallback = 0;
  long long routed_iterations = 0;
  // with profiling on (router_set_profiling), CUDA-event milliseconds of the routed assignment's
  // stages summed over the routed iterations: [0] center separation, [1] centers in group order,
  // [2] network inference, [3] sort by group, [4] group scan, [5] in-group near ties (candidate
  // pass and resolve), [6] certificate
  double stage_ms[7] = {0, 0, 0, 0, 0, 0, 0};
};

// groups: G; hidden: H; split: the tier has the BF16 residual planes of the centers.
cudaError_t router_create(Router** r, const RouterIO& io, int groups, int hidden, bool split,
                          cudaStream_t s);
void router_destroy(Router* r, cudaStream_t s);
bool router_trained(const Router* r);
// (Re)trains on the current labels (those of the last assignment, for the current centers):
// forms the groups of centers on the first call, draws a training sample, trains the network,
// and refreshes its tensor-core copy. Host-synchronous.
cudaError_t router_train(Router* r, const RouterIO& io, cudaStream_t s);
// Routes every point, scans each routed point's group of centers on the tensor cores (exact
// within the group), and certifies the group's winner as the arg-min over all centers when
// 2 d(x, c*) < min over centers c outside the group of d(c*, c) (computed for the current
// centers: io.Cop / io.cn must belong to them). Certified points get their
// label in io.labels; the others are listed in fb_list / *fb_count (device) for the full scan.
cudaError_t router_assign(Router* r, const RouterIO& io, int* fb_list, int* fb_count,
                          cudaStream_t s);
// The points of fb_list (count on the device, at most cap) as a compact data set for the full
// scan, and the compact labels back to their points.
cudaError_t router_gather_fallback(const int* fb_list, const int* fb_count, long long cap,
                                   const float* X, long long ldx, const float* xn, const void* Xb,
                                   const void* Xl, long long ldb, float* XF, float* xnF, void* XbF,
                                   void* XlF, const int* stop, cudaStream_t s);
cudaError_t router_scatter_labels(const int* fb_list, const int* fb_count, long long cap,
                                  const int* labF, int* labels, const int* stop, cudaStream_t s);
// Host copy of the statistics (reads the device counters; synchronises s).
cudaError_t router_stats(Router* r, RouterStats* out, cudaStream_t s);
size_t router_device_bytes(const Router* r);
// Stage timing of the routed assignment (CUDA events on its stream).
void router_set_profiling(Router* r, bool on);

}  // namespace kmgb
