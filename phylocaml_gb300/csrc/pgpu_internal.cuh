// Internal declarations shared by the translation units of libphylo_gpu.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>

#include "../../include/phylo_gpu.h"

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------

enum {
  BUF_TIPS = 0,
  BUF_WEIGHTS,
  BUF_OUT,
  BUF_SITECOST,
  BUF_OPS,
  BUF_TIPSEQ,
  BUF_SCALAR,
  BUF_A,
  BUF_B,
  BUF_C,
  BUF_D,
  BUF_E,
  BUF_F,
  BUF_G,
  BUF_H,
  BUF_I,
  BUF_J,
  BUF_SPLIT,
  BUF_COUNT
};

// One internal-node step of a stack-machine postorder.  `a` is evaluated
// first, `b` second; a child id >= n_tips lives on the stack (b above a when
// both are internal), a tip id is read from the tip rows.  `k` is the
// internal index of the node (its output row).
struct SchedOp {
  int32_t k, a, b, pad;
};

struct TreeSchedule {
  int32_t n_tips = 0;
  std::vector<SchedOp> ops;        // evaluation order
  std::vector<int32_t> tip_seq;    // tips in the order the ops read them
  int max_depth = 0;               // largest stack height reached
};

// The postorder cut into disjoint subtrees (segments), each a stack-machine
// schedule of its own, dealt to the warps of a CTA, plus the few nodes above
// them (top).  Segment ops read tips from their own tip sequence and
// internal children from their own stack; a top op's child reference is a
// tip id (>= 0), a segment result (-1 - (warp * 32 + row)) or an earlier
// top result (-1000 - t).
struct SplitSchedule {
  int n_seg = 0, rows = 0;     // rows: ring + stack rows one warp needs
  std::vector<int4> ops;       // segment ops, segments one after another
  std::vector<int32_t> tips;   // segment tip sequences, one after another
  std::vector<int4> seg;       // {op_off, n_ops, tip_off, n_tips}, by warp
  std::vector<int4> wseg;      // per warp {first segment, count, 0, 0}
  std::vector<int4> top;       // {k, ref_a, ref_b, 0} in postorder
};

// column chunks (at most) of the host-buffer calls' copies: 2-D copies of
// narrower columns overlap each other worse
constexpr int PGPU_COPY_CHUNKS = 4;

struct pgpu_ctx {
  int device = 0;
  int num_sms = 0;
  int cc_major = 0, cc_minor = 0;
  size_t smem_optin = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::string err;
  uint64_t launches = 0;
  void *buf[BUF_COUNT] = {};
  size_t cap[BUF_COUNT] = {};
  int *d_flag = nullptr;       // device error word written by bounded waits
  void *h_pinned = nullptr;    // small pinned staging area for scalars
  // the last tree scheduled, kept on the device (BUF_OPS, BUF_TIPSEQ) so
  // repeated calls on one tree upload nothing
  bool sched_valid = false;
  std::vector<int32_t> sched_left, sched_right;
  TreeSchedule sched;
  // the last tree's segment schedule, resident in BUF_SPLIT
  bool split_valid = false;
  std::vector<int32_t> split_left, split_right;
  SplitSchedule split;
  // double-buffered pinned staging of small per-call parameters
  void *stage_h[2] = {};
  void *stage_d[2] = {};
  size_t stage_cap[2] = {};
  cudaEvent_t stage_ev[2] = {};
  int stage_next = 0, stage_cur = 0;
  // words of a state-set row per CTA of the Fitch tree kernel (0: picked
  // per launch)
  int fitch_tile_words = 0;
  // streams for host-to-device and device-to-host copies that overlap the
  // kernels of host-buffer calls, with one event per copied chunk, one for
  // the start of a call and one per finished chunk
  cudaStream_t copy_stream = nullptr, d2h_stream = nullptr;
  cudaEvent_t copy_ev[PGPU_COPY_CHUNKS + 1] = {};
  cudaEvent_t done_ev[PGPU_COPY_CHUNKS] = {};
  // a second stream for launches that may run beside the context stream's
  // (the next chunk's CTAs fill SMs as the previous chunk's drain), with
  // the events that fork it from and join it to the context stream
  cudaStream_t aux_stream = nullptr;
  cudaEvent_t aux_ev[2] = {};
};

// Creates the copy streams, the auxiliary stream and their events on first use.
pgpu_status pgpu_copy_stream(pgpu_ctx *ctx);
// A host-buffer call that fails after queueing chunk copies waits for them
// before returning, so no copy touches the caller's buffers afterwards.
pgpu_status pgpu_settle_copies(pgpu_ctx *ctx, pgpu_status st);
// The device's address of p when p lies in page-locked host memory the
// device can reach (cudaMallocHost, cudaHostAlloc, cudaHostRegister), else
// null: kernels may then read and write the caller's buffer over the
// CPU-GPU link directly.
void *pgpu_host_view(const void *p);

// Rows of a host-buffer tree call still in host memory: the tip rows go to
// the device buffer and the node rows come back column chunk by column
// chunk on the copy streams, overlapping the kernels.
struct HostRows {
  const uint32_t *tips;   // [n_tips][n_words]
  uint32_t *node_sets;    // [n_tips - 1][n_words]
};

pgpu_status pgpu_set_err(pgpu_ctx *ctx, pgpu_status st, const char *fmt, ...);

#define PGPU_CUDA(ctx, call)                                                        \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess) {                                                        \
      (void)cudaGetLastError();                                                     \
      return pgpu_set_err((ctx),                                                    \
                          e_ == cudaErrorMemoryAllocation ? PGPU_ERR_OOM : PGPU_ERR_CUDA, \
                          "%s failed: %s", #call, cudaGetErrorString(e_));          \
    }                                                                               \
  } while (0)

#define PGPU_TRY(expr)                \
  do {                                \
    pgpu_status s_ = (expr);          \
    if (s_ != PGPU_OK) return s_;     \
  } while (0)

// Grow-only device buffer owned by the context.
pgpu_status pgpu_buf(pgpu_ctx *ctx, int slot, size_t bytes, void **out);
// Launch bookkeeping: checks the launch error and counts it.
pgpu_status pgpu_after_launch(pgpu_ctx *ctx, const char *what);
// Reads and clears the device error word after a synchronize.
pgpu_status pgpu_check_flag(pgpu_ctx *ctx, const char *what);
// Pinned host block and its device twin for `bytes` of small parameters;
// fill *host, then pgpu_stage_commit copies it on the context's stream.
// Two blocks alternate, so the host only waits for the copy issued two
// calls earlier.
pgpu_status pgpu_stage(pgpu_ctx *ctx, size_t bytes, void **host, void **dev);
pgpu_status pgpu_stage_commit(pgpu_ctx *ctx, size_t bytes);

// ---------------------------------------------------------------------------
// tree schedule (schedule.cpp)
// ---------------------------------------------------------------------------

pgpu_status pgpu_build_schedule(pgpu_ctx *ctx, const pgpu_tree *tree, TreeSchedule *out);
// Builds (or reuses) the schedule of `tree` and makes its ops and tip
// sequence resident on the device.
pgpu_status pgpu_schedule_device(pgpu_ctx *ctx, const pgpu_tree *tree, const TreeSchedule **sch,
                                 const int4 **d_ops, const int32_t **d_tip_seq);

// The cost-matrix postorder on the Fitch kernel's segmented schedule
// (fitch.cu); *launched is false when the tree does not fit its shared
// memory.
pgpu_status pgpu_tcm_tree_split(pgpu_ctx *ctx, const pgpu_tree *tree, const uint32_t *tips,
                                size_t ld, const uint32_t *weights, size_t n_sites,
                                const uint32_t *table_dev, int flush_period, uint32_t *node_sets,
                                uint32_t *site_cost, unsigned long long *total, bool *launched,
                                const HostRows *io = nullptr);

// ---------------------------------------------------------------------------
// device helpers: mbarrier, bulk copies, bounded waits
// ---------------------------------------------------------------------------

#define PGPU_FLAG_TIMEOUT 1
#define PGPU_FLAG_BADCODE 2
#define PGPU_FLAG_NAN 4
#define PGPU_FLAG_NONREV 8
#define PGPU_FLAG_EIGEN 16

// error-word bit of a model status (PGPU_ERR_NAN / _NONREVERSIBLE / _EIGEN)
__host__ __device__ inline int pgpu_model_flag(int st) {
  return st == PGPU_ERR_NAN ? PGPU_FLAG_NAN
                            : st == PGPU_ERR_NONREVERSIBLE ? PGPU_FLAG_NONREV : PGPU_FLAG_EIGEN;
}
#define PGPU_WAIT_NS 2000000000ull   // 2 s budget for any single device wait

#ifdef __CUDACC__
__device__ __forceinline__ uint64_t pgpu_globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void fence_mbarrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile(
      "{\n\t.reg .b64 st;\n\t"
      "mbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile(
      "{\n\t.reg .b64 st;\n\t"
      "mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(smem_u32(bar)),
      "r"(bytes)
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Waits for phase `parity` of *bar to complete.  Gives up after
// PGPU_WAIT_NS, raising PGPU_FLAG_TIMEOUT in *flag, and returns false.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, int *flag) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = pgpu_globaltimer();
  uint32_t it = 0;
  while (!mbar_try_wait(bar, parity)) {
    if ((++it & 255u) == 0u) {
      if (pgpu_globaltimer() - t0 > PGPU_WAIT_NS) {
        atomicOr(flag, PGPU_FLAG_TIMEOUT);
        return false;
      }
      if (*(volatile int *)flag & PGPU_FLAG_TIMEOUT) return false;
    }
  }
  return true;
}

// As mbar_try_wait, but a thread whose phase is not complete may stay
// suspended for up to `ns` nanoseconds (it resumes as soon as the phase
// completes), so a long wait costs few retries.
__device__ __forceinline__ bool mbar_try_wait_for(uint64_t *bar, uint32_t parity, uint32_t ns) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity), "r"(ns)
      : "memory");
  return ok != 0;
}

// mbar_wait_bounded with suspended retries: the same PGPU_WAIT_NS budget,
// the clock read every 16 retries.
__device__ __forceinline__ bool mbar_wait_bounded_for(uint64_t *bar, uint32_t parity, int *flag,
                                                      uint32_t ns = 20000u) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = pgpu_globaltimer();
  uint32_t it = 0;
  while (!mbar_try_wait_for(bar, parity, ns)) {
    if ((++it & 15u) == 0u) {
      if (pgpu_globaltimer() - t0 > PGPU_WAIT_NS) {
        atomicOr(flag, PGPU_FLAG_TIMEOUT);
        return false;
      }
      if (*(volatile int *)flag & PGPU_FLAG_TIMEOUT) return false;
    }
  }
  return true;
}

// 1-D bulk copy global -> shared, completion signalled on *bar.
// dst, src and bytes must be multiples of 16.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes,
                                         uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
#endif
