// Fitch postorder for callers that cannot allocate device memory.
//
// pgpu_fitch_tree and pgpu_fitch_tree_dev keep their scratch (the stack
// schedule of the tree and an error word) in buffers the context obtains with
// cudaMalloc.  Some callers cannot allow that: a host program that hands all
// of the GPU's memory to its own pool up front, or a service that forbids
// allocation once it is serving (cudaMalloc can synchronise the device and
// stall every other stream).  pgpu_fitch_tree_noalloc serves them: it needs
// no context and allocates nothing.  Its scratch is the one file-scope device
// array below, of fixed size, which every GPU that loads this library holds
// until the process exits.
//
// Limits and sharing:
//   - trees of at most PGPU_NOALLOC_MAX_TIPS tips (larger ones get
//     PGPU_ERR_LIMIT);
//   - every call uses the same array and leaves the last call's schedule in
//     it; the error word is cleared at the start of each call.  Calls whose
//     work overlaps on the GPU (different streams, or different host threads
//     on one device) race on the array and must be serialised by the caller;
//     host threads are serialised here while the schedule is written.
//   - the call copies the schedule from host memory, reads the error word
//     back and waits for the stream before it returns.
//   - the first call in a device's context looks up the array's device
//     address with cudaGetSymbolAddress (with that device current) and keeps
//     it for that context, so make that first call before any stream capture
//     begins.  A device reset between calls is not supported: a new context
//     can reuse the old one's handle, and the kept address would be stale.
#include <algorithm>
#include <mutex>

#include "pgpu_internal.cuh"

pgpu_status pgpu_fitch_tree_launch_raw(cudaStream_t stream, const int4 *ops, const int32_t *tip_seq,
                                       int n_ops, int depth, int *flag, int32_t n_tips,
                                       const uint32_t *tips, size_t ld, const uint32_t *weights,
                                       size_t n_sites, int lb, uint32_t *node_sets,
                                       uint32_t *site_cost, uint64_t *total);

#define PGPU_NOALLOC_MAX_TIPS 16384

namespace {

constexpr int kMaxTips = PGPU_NOALLOC_MAX_TIPS;
// layout of the scratch array, in int4 units: the schedule ops, then the tip
// sequence (4 ids per int4), then the error word
constexpr int kOpsAt = 0;
constexpr int kSeqAt = kMaxTips;                 // ops need kMaxTips - 1 entries
constexpr int kFlagAt = kSeqAt + kMaxTips / 4;
constexpr int kScratchInt4 = kFlagAt + 16;       // 20,496 int4 = 327,936 bytes

static __device__ __align__(256) int4 g_noalloc_scratch[kScratchInt4];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
// per device: the context the address was looked up in, and the address
struct ScratchSlot {
  void *context;
  void *addr;
};
ScratchSlot g_scratch[kMaxDevices] = {};

// The calling thread's current context (a CUcontext), through the driver's
// cuCtxGetCurrent reached from the runtime, so the library needs no link
// against the driver library.  Null if there is none yet.
void *current_context() {
  using CtxGetCurrent = int (*)(void **);
  static CtxGetCurrent fn = nullptr;   // guarded by g_mutex
  if (!fn) {
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    void *f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !f) {
      (void)cudaGetLastError();
      return nullptr;
    }
    fn = reinterpret_cast<CtxGetCurrent>(f);
  }
  void *c = nullptr;
  return fn(&c) == 0 ? c : nullptr;
}

// host-side schedule workspace, also fixed (no heap), guarded by g_mutex
int32_t h_uses[2 * kMaxTips], h_need[2 * kMaxTips];
uint8_t h_swap[kMaxTips];
int32_t h_dfs_node[2 * kMaxTips];
uint8_t h_dfs_phase[2 * kMaxTips];
int32_t h_sim[kMaxTips];
int4 h_ops[kMaxTips];
int32_t h_seq[kMaxTips];

// Sethi-Ullman stack schedule of the tree (the order fitch_tree_kernel
// expects: a evaluated first, b second, b above a on the stack).
pgpu_status schedule_static(const pgpu_tree *t, int *depth_out) {
  const int32_t n = t->n_tips, n_int = n - 1, n_nodes = 2 * n - 1;
  std::fill(h_uses, h_uses + n_nodes, 0);
  for (int32_t k = 0; k < n_int; ++k) {
    const int32_t a = t->left[k], b = t->right[k];
    if (a < 0 || b < 0 || a >= n + k || b >= n + k || a == b) return PGPU_ERR_ARG;
    h_uses[a]++;
    h_uses[b]++;
  }
  for (int32_t id = 0; id < n_nodes - 1; ++id)
    if (h_uses[id] != 1) return PGPU_ERR_ARG;
  std::fill(h_need, h_need + n_nodes, 0);
  for (int32_t k = 0; k < n_int; ++k) {
    const int32_t a = t->left[k], b = t->right[k];
    const int32_t ha = a >= n, hb = b >= n;
    const int32_t a_first = std::max(h_need[a], ha + h_need[b]);
    const int32_t b_first = std::max(h_need[b], hb + h_need[a]);
    h_swap[k] = b_first < a_first;
    h_need[n + k] = std::max(std::min(a_first, b_first), 1);
  }
  int top = 0, n_ops = 0, n_seq = 0;
  h_dfs_node[top] = n_nodes - 1;
  h_dfs_phase[top++] = 0;
  while (top > 0) {
    --top;
    const int32_t v = h_dfs_node[top], k = v - n;
    int32_t first = t->left[k], second = t->right[k];
    if (h_swap[k]) std::swap(first, second);
    if (h_dfs_phase[top] == 0) {
      h_dfs_phase[top++] = 1;   // v stays, now in its second phase
      if (second >= n) {
        h_dfs_node[top] = second;
        h_dfs_phase[top++] = 0;
      }
      if (first >= n) {
        h_dfs_node[top] = first;
        h_dfs_phase[top++] = 0;
      }
    } else {
      h_ops[n_ops++] = make_int4(k, first, second, 0);
    }
  }
  int sp = 0, depth = 0;
  for (int i = 0; i < n_ops; ++i) {
    const int4 op = h_ops[i];
    if (op.z >= n) {
      if (sp == 0 || h_sim[sp - 1] != op.z) return PGPU_ERR_ARG;
      --sp;
    }
    if (op.y >= n) {
      if (sp == 0 || h_sim[sp - 1] != op.y) return PGPU_ERR_ARG;
      --sp;
    }
    if (op.y < n) h_seq[n_seq++] = op.y;
    if (op.z < n) h_seq[n_seq++] = op.z;
    h_sim[sp++] = n + op.x;
    depth = std::max(depth, sp);
  }
  if (n_ops != n_int || n_seq != n || sp != 1) return PGPU_ERR_ARG;
  *depth_out = depth;
  return PGPU_OK;
}

}  // namespace

extern "C" pgpu_status pgpu_fitch_tree_noalloc(const pgpu_tree *tree, const uint32_t *tips_dev,
                                               size_t ld_words, const uint32_t *weights_dev,
                                               size_t n_sites, int lane_bits,
                                               uint32_t *node_sets_dev, uint32_t *site_cost_dev,
                                               uint64_t *total_dev, void *cuda_stream) {
  if (!tree || !tree->left || !tree->right || tree->n_tips < 2) return PGPU_ERR_ARG;
  if (tree->n_tips > kMaxTips) return PGPU_ERR_LIMIT;
  cudaStream_t stream = static_cast<cudaStream_t>(cuda_stream);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    (void)cudaGetLastError();
    return PGPU_ERR_CUDA;
  }
  std::lock_guard<std::mutex> lock(g_mutex);
  // set-up, once per device and context, with that device current: the
  // array's name is a host-side stand-in, so the device address must be
  // looked up (which also creates the device's primary context if needed)
  ScratchSlot &slot = g_scratch[dev];
  void *context = current_context();
  if (!slot.addr || !context || slot.context != context) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
      (void)cudaGetLastError();
      return PGPU_ERR_CUDA;
    }
    slot.addr = p;
    slot.context = context ? context : current_context();
  }
  int4 *scratch = static_cast<int4 *>(slot.addr);
  int depth = 0;
  PGPU_TRY(schedule_static(tree, &depth));
  const int n = tree->n_tips;
  int4 *d_ops = scratch + kOpsAt;
  int32_t *d_seq = reinterpret_cast<int32_t *>(scratch + kSeqAt);
  int *d_flag = reinterpret_cast<int *>(scratch + kFlagAt);
  // pageable-source copies return once the source has been staged, so the
  // static host workspace may be rewritten by the next call
  if (cudaMemcpyAsync(d_ops, h_ops, sizeof(int4) * (size_t)(n - 1), cudaMemcpyHostToDevice,
                      stream) != cudaSuccess ||
      cudaMemcpyAsync(d_seq, h_seq, sizeof(int32_t) * (size_t)n, cudaMemcpyHostToDevice, stream) !=
          cudaSuccess ||
      cudaMemsetAsync(d_flag, 0, sizeof(int), stream) != cudaSuccess) {
    (void)cudaGetLastError();
    return PGPU_ERR_CUDA;
  }
  PGPU_TRY(pgpu_fitch_tree_launch_raw(stream, d_ops, d_seq, n - 1, depth, d_flag, n, tips_dev,
                                      ld_words, weights_dev, n_sites, lane_bits, node_sets_dev,
                                      site_cost_dev, total_dev));
  int flag = 0;
  if (cudaMemcpyAsync(&flag, d_flag, sizeof(int), cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
      cudaStreamSynchronize(stream) != cudaSuccess) {
    (void)cudaGetLastError();
    return PGPU_ERR_CUDA;
  }
  return flag ? PGPU_ERR_TIMEOUT : PGPU_OK;
}
