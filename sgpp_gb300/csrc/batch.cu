// Batched, continuously refilled regression-fit engine (C ABI sgmev_batch_* in sgmev.h).
//
// A batch owns device pools for up to `max_slots` independent problems (grid, data, K right-hand
// sides, CG state). Every problem runs the mixed-precision fit of sgmev_fit as a device-side
// state machine:
//
//   phase OUTER  r = b - A x with the df64 (FP64-accurate) kernels; if ||r_c||^2 <= eps^2 r0_c for
//                every column c (or the outer cap is hit) -> DONE, else start an inner solve
//   phase INNER  one CG iteration on A dx = r with FP32 kernels and FP64 vectors per step, every
//                column with its own scalars; when all columns reach the inner tolerance (or the
//                inner cap) -> x += dx and back to OUTER
//
// One step = a fixed sequence of launches over all slots (each kernel skips slots in other
// phases), captured once into a CUDA graph and replayed; the host reads the per-slot phases after
// each step and admits new problems into free slots (continuous batching). Problems never
// interact: every item of every launch reads and writes only its own slot's buffers.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/sgmev.h"
#include "batch_kernels.cuh"

namespace sgmev {
extern thread_local std::string g_last_error;
}

namespace {

using namespace sgmev;

int bfail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

#define B_CUDA(call)                                                                          \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess)                                                                    \
      return bfail(e_ == cudaErrorMemoryAllocation ? SGMEV_ERR_OOM : SGMEV_ERR_CUDA,          \
                   std::string(#call) + ": " + cudaGetErrorString(e_));                       \
  } while (0)
#define B_TRY(expr)                      \
  do {                                   \
    int rc_ = (expr);                    \
    if (rc_ != SGMEV_OK) return rc_;     \
  } while (0)

enum Phase { PH_EMPTY = 0, PH_OUTER = 1, PH_INNER = 2, PH_DONE = 3 };

constexpr int kMaxBatchDim = 16;
constexpr int kSegLen = 4096;   // elements per elementwise segment item

int64_t cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }
int64_t rup(int64_t a, int64_t b) { return cdiv(a, b) * b; }

// per (slot, column) CG scalars, device-resident
struct ColState {
  double r0;        // ||b - A x0||^2 at the first outer step
  double rnorm2;    // ||r||^2 of the latest outer residual
  double delta;     // inner r.r
  double delta0;    // inner stopping threshold
  double dq;        // inner d.q
  double a;         // inner step length of the current iteration
  int inner_done;   // column reached the inner tolerance
  int outer_done;   // column reached the outer tolerance
};

struct SlotCtl {    // per-slot control, device-resident
  int phase;
  int inner_it;     // iterations of the current inner solve
  int total_it;     // inner iterations so far
  int outer_it;     // outer residual evaluations so far
  int start_inner;  // set by the outer decision: initialise the inner vectors this step
  int finish_inner; // set by the inner decision: x += dx this step
  double eps;       // outer relative tolerance
  double eps_inner; // inner relative tolerance
  int max_it;       // inner iteration budget of the whole fit
  double lm;        // lambda * M
};

struct Seg {
  int slot;
  int64_t begin, end;
};

// ---------------------------------------------------------------------------------------
// persistent tile kernels
// ---------------------------------------------------------------------------------------
template <class Pol, int K>
__global__ void __launch_bounds__(kBB) batch_mult_kernel(
    const BatchSlot* __restrict__ slots, const SlotCtl* __restrict__ ctl, int want_phase,
    const BatchItem* __restrict__ items, int n_items, int* __restrict__ counter,
    const float* __restrict__ xh, const float* __restrict__ xl, const float2* __restrict__ li,
    const float4* __restrict__ gq, const float* __restrict__ ah, const float* __restrict__ al,
    float2* __restrict__ part) {
  __shared__ float2 s_li[kBGT * kMaxBatchDim];
  __shared__ float4 s_gq[IsDF<Pol>::value ? kBGT * kMaxBatchDim : 1];
  __shared__ float s_ah[kBGT * K];
  __shared__ float s_al[IsDF<Pol>::value ? kBGT * K : 1];
  __shared__ int s_item;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_item = atomicAdd(counter, 1);
    __syncthreads();
    const int i = s_item;
    if (i >= n_items) break;
    const BatchItem it = items[i];
    if (ctl[it.slot].phase != want_phase) continue;
    const BatchSlot s = slots[it.slot];
    switch (s.dim) {
#define D_CASE(D)                                                                           \
  case D:                                                                                   \
    batch_mult_item<Pol, D, K>(s, it, xh, xl, li, gq, ah, al, part, s_li, s_gq, s_ah, s_al); \
    break;
      D_CASE(1) D_CASE(2) D_CASE(3) D_CASE(4) D_CASE(5) D_CASE(6) D_CASE(7) D_CASE(8)
      D_CASE(9) D_CASE(10) D_CASE(11) D_CASE(12) D_CASE(13) D_CASE(14) D_CASE(15) D_CASE(16)
#undef D_CASE
      default:
        break;
    }
  }
}

template <class Pol, int K>
__global__ void __launch_bounds__(kBB) batch_multt_kernel(
    const BatchSlot* __restrict__ slots, const SlotCtl* __restrict__ ctl, int want_phase,
    const BatchItem* __restrict__ items, int n_items, int* __restrict__ counter,
    const float* __restrict__ xh, const float* __restrict__ xl, const float2* __restrict__ li,
    const float4* __restrict__ gq, const float* __restrict__ vh, const float* __restrict__ vl,
    float2* __restrict__ part) {
  __shared__ float s_xh[kMaxBatchDim * kBDT];
  __shared__ float s_xl[IsDF<Pol>::value ? kMaxBatchDim * kBDT : 1];
  __shared__ float s_vh[kBDT * K];
  __shared__ float s_vl[IsDF<Pol>::value ? kBDT * K : 1];
  __shared__ int s_item;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_item = atomicAdd(counter, 1);
    __syncthreads();
    const int i = s_item;
    if (i >= n_items) break;
    const BatchItem it = items[i];
    if (ctl[it.slot].phase != want_phase) continue;
    const BatchSlot s = slots[it.slot];
    switch (s.dim) {
#define D_CASE(D)                                                                               \
  case D:                                                                                       \
    batch_multt_item<Pol, D, K>(s, it, xh, xl, li, gq, vh, vl, part, s_xh, s_xl, s_vh, s_vl);   \
    break;
      D_CASE(1) D_CASE(2) D_CASE(3) D_CASE(4) D_CASE(5) D_CASE(6) D_CASE(7) D_CASE(8)
      D_CASE(9) D_CASE(10) D_CASE(11) D_CASE(12) D_CASE(13) D_CASE(14) D_CASE(15) D_CASE(16)
#undef D_CASE
      default:
        break;
    }
  }
}

// ---------------------------------------------------------------------------------------
// segment-wise kernels (each CTA walks segment items; a segment lies inside one slot)
// ---------------------------------------------------------------------------------------
#define SEG_LOOP(segs, nseg)                                                        \
  for (int si = blockIdx.x; si < (nseg); si += gridDim.x)                           \
    if (const Seg sg = (segs)[si]; true)                                            \
      for (int64_t e = sg.begin + threadIdx.x; e < sg.end; e += blockDim.x)

// FP64 N-vector -> FP32 hi (and lo) for the tile kernels, slots in `want_phase`
__global__ void b_split_kernel(const Seg* __restrict__ segs, int nseg, const SlotCtl* __restrict__ ctl,
                               int want_phase, const double* __restrict__ src,
                               float* __restrict__ hi, float* __restrict__ lo) {
  SEG_LOOP(segs, nseg) {
    if (ctl[sg.slot].phase != want_phase) break;
    const double v = src[e];
    const float h = static_cast<float>(v);
    hi[e] = h;
    if (lo) lo[e] = static_cast<float>(v - static_cast<double>(h));
  }
}

// reduce mult partials over grid chunks -> M-side FP32 (hi, lo) input of multT; rows >= m are 0
__global__ void b_reduce_m_kernel(const Seg* __restrict__ segs, int nseg, const SlotCtl* __restrict__ ctl,
                                  int want_phase, const BatchSlot* __restrict__ slots, int K,
                                  int list, const float2* __restrict__ part,
                                  float* __restrict__ vh, float* __restrict__ vl) {
  SEG_LOOP(segs, nseg) {
    if (ctl[sg.slot].phase != want_phase) break;
    const BatchSlot s = slots[sg.slot];
    const int64_t local = e - s.mvec_off;  // element within the slot: row * K + c
    double acc = 0.0;
    if (local / K < s.m) {
      for (int q = 0; q < s.nchunk[list]; ++q) {
        const float2 p = part[s.part_off + static_cast<int64_t>(q) * s.mpad * K + local];
        acc += static_cast<double>(p.x) + static_cast<double>(p.y);
      }
    }
    const float h = static_cast<float>(acc);
    vh[e] = h;
    if (vl) vl[e] = static_cast<float>(acc - static_cast<double>(h));
  }
}

// reduce multT partials over data chunks: out = sum + lm * add (FP64); rows >= n are 0
__global__ void b_reduce_n_kernel(const Seg* __restrict__ segs, int nseg, const SlotCtl* __restrict__ ctl,
                                  int want_phase, const BatchSlot* __restrict__ slots, int K,
                                  int list, const float2* __restrict__ part,
                                  const double* __restrict__ add, double* __restrict__ out) {
  SEG_LOOP(segs, nseg) {
    if (ctl[sg.slot].phase != want_phase) break;
    const BatchSlot s = slots[sg.slot];
    const int64_t local = e - s.nvec_off;
    double acc = 0.0;
    if (local / K < s.n) {
      for (int q = 0; q < s.nchunk[list]; ++q) {
        const float2 p = part[s.part_off + static_cast<int64_t>(q) * s.npad * K + local];
        acc += static_cast<double>(p.x) + static_cast<double>(p.y);
      }
      if (add) acc = fma(ctl[sg.slot].lm, add[e], acc);
    }
    out[e] = acc;
  }
}

// per-slot, per-column dot products (deterministic): one CTA per slot, blockDim % K == 0
template <int K>
__global__ void b_dot_kernel(const BatchSlot* __restrict__ slots, const SlotCtl* __restrict__ ctl,
                             int want_phase, const double* __restrict__ a, const double* __restrict__ b,
                             double* __restrict__ out /* [slot * K + c] */) {
  __shared__ double s[256];
  const int slot = blockIdx.x;
  if (ctl[slot].phase != want_phase) return;
  const BatchSlot sl = slots[slot];
  double acc = 0.0;
  const int64_t total = sl.npad * K;
  for (int64_t e = threadIdx.x; e < total; e += blockDim.x)
    acc = fma(a[sl.nvec_off + e], b[sl.nvec_off + e], acc);
  s[threadIdx.x] = acc;
  __syncthreads();
  // threads t and t + w share the column when w is a multiple of K
  for (int w = blockDim.x / 2; w >= K; w >>= 1) {
    if (threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < K) out[slot * K + threadIdx.x] = s[threadIdx.x];
}

// ---------------------------------------------------------------------------------------
// state machine kernels
// ---------------------------------------------------------------------------------------
// after the outer residual dot (rnorm2 in dots[]): decide DONE or start an inner solve
template <int K>
__global__ void b_outer_decide_kernel(int nslots, SlotCtl* __restrict__ ctl,
                                      ColState* __restrict__ col, const double* __restrict__ dots,
                                      int max_outer) {
  const int slot = blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= nslots) return;
  SlotCtl& c = ctl[slot];
  c.start_inner = 0;
  if (c.phase != PH_OUTER) return;
  bool all = true;
  for (int k = 0; k < K; ++k) {
    ColState& s = col[slot * K + k];
    const double r = dots[slot * K + k];
    if (c.outer_it == 0) s.r0 = r;
    s.rnorm2 = r;
    s.outer_done = (r <= c.eps * c.eps * s.r0) || r == 0.0;
    all = all && s.outer_done;
    // inner solve start: delta = r.r, tolerance relative to it
    s.delta = r;
    const double want = fmax(c.eps_inner, fmin(0.5, c.eps * sqrt(s.r0 / fmax(r, 1e-300)) * 0.5));
    s.delta0 = r * want * want;
    s.inner_done = s.outer_done || r == 0.0;
  }
  c.outer_it += 1;
  if (all || c.outer_it >= max_outer || c.total_it >= c.max_it) {
    c.phase = PH_DONE;
  } else {
    c.phase = PH_INNER;
    c.inner_it = 0;
    c.start_inner = 1;
  }
}

// inner-solve vector initialisation for slots that just entered INNER: dx = 0, r = rr, d = rr
__global__ void b_start_inner_kernel(const Seg* __restrict__ segs, int nseg, const SlotCtl* __restrict__ ctl,
                                     const double* __restrict__ rr, double* __restrict__ dx,
                                     double* __restrict__ r, double* __restrict__ d) {
  SEG_LOOP(segs, nseg) {
    if (!ctl[sg.slot].start_inner) break;
    dx[e] = 0.0;
    r[e] = rr[e];
    d[e] = rr[e];
  }
}

// step length a = delta / (d.q) per column (0 for finished columns)
template <int K>
__global__ void b_inner_alpha_kernel(int nslots, const SlotCtl* __restrict__ ctl,
                                     ColState* __restrict__ col, const double* __restrict__ dots) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nslots * K) return;
  const int slot = i / K;
  ColState& s = col[i];
  if (ctl[slot].phase != PH_INNER) return;
  s.dq = dots[i];
  s.a = (!s.inner_done && s.dq != 0.0) ? s.delta / s.dq : 0.0;
  if (s.dq == 0.0) s.inner_done = 1;
}

// dx += a d, r -= a q
template <int K>
__global__ void b_inner_update_kernel(const Seg* __restrict__ segs, int nseg,
                                      const SlotCtl* __restrict__ ctl,
                                      const ColState* __restrict__ col,
                                      const BatchSlot* __restrict__ slots, const double* __restrict__ d,
                                      const double* __restrict__ q, double* __restrict__ dx,
                                      double* __restrict__ r) {
  SEG_LOOP(segs, nseg) {
    if (ctl[sg.slot].phase != PH_INNER) break;
    const int c = static_cast<int>((e - slots[sg.slot].nvec_off) % K);
    const double a = col[sg.slot * K + c].a;
    dx[e] = fma(a, d[e], dx[e]);
    r[e] = fma(-a, q[e], r[e]);
  }
}

// new delta from r.r; beta; decide inner completion per slot
template <int K>
__global__ void b_inner_decide_kernel(int nslots, SlotCtl* __restrict__ ctl,
                                      ColState* __restrict__ col, const double* __restrict__ dots,
                                      int max_inner, double* __restrict__ beta_out) {
  const int slot = blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= nslots) return;
  SlotCtl& c = ctl[slot];
  c.finish_inner = 0;
  if (c.phase != PH_INNER) return;
  bool all = true;
  for (int k = 0; k < K; ++k) {
    ColState& s = col[slot * K + k];
    const double dn = dots[slot * K + k];
    double beta = 0.0;
    if (!s.inner_done) {
      beta = s.delta > 0.0 ? dn / s.delta : 0.0;
      s.delta = dn;
      if (dn <= s.delta0) s.inner_done = 1;
    }
    beta_out[slot * K + k] = beta;
    all = all && s.inner_done;
  }
  c.inner_it += 1;
  c.total_it += 1;
  if (all || c.inner_it >= max_inner || c.total_it >= c.max_it) {
    c.finish_inner = 1;
    c.phase = PH_OUTER;
  }
}

// d = r + beta d for continuing slots; x += dx for slots that finished their inner solve
template <int K>
__global__ void b_inner_tail_kernel(const Seg* __restrict__ segs, int nseg,
                                    const SlotCtl* __restrict__ ctl,
                                    const BatchSlot* __restrict__ slots,
                                    const double* __restrict__ beta, const double* __restrict__ r,
                                    double* __restrict__ d, const double* __restrict__ dx,
                                    double* __restrict__ x) {
  SEG_LOOP(segs, nseg) {
    const SlotCtl& c = ctl[sg.slot];
    if (c.finish_inner) {
      x[e] += dx[e];
    } else if (c.phase == PH_INNER) {
      const int k = static_cast<int>((e - slots[sg.slot].nvec_off) % K);
      d[e] = fma(beta[sg.slot * K + k], d[e], r[e]);
    } else {
      break;
    }
  }
}

// rr = b - q (outer residual)
__global__ void b_residual_kernel(const Seg* __restrict__ segs, int nseg, const SlotCtl* __restrict__ ctl,
                                  const double* __restrict__ b, const double* __restrict__ q,
                                  double* __restrict__ rr) {
  SEG_LOOP(segs, nseg) {
    if (ctl[sg.slot].phase != PH_OUTER) break;
    rr[e] = b[e] - q[e];
  }
}

// ---------------------------------------------------------------------------------------
// first-fit range allocator for the device pools (host-side bookkeeping)
// ---------------------------------------------------------------------------------------
class RangeAlloc {
 public:
  explicit RangeAlloc(int64_t cap = 0) : cap_(cap) {}
  bool alloc(int64_t n, int64_t* off) {
    int64_t pos = 0;
    for (size_t k = 0; k <= used_.size(); ++k) {
      const int64_t next = k < used_.size() ? used_[k].first : cap_;
      if (next - pos >= n) {
        used_.insert(used_.begin() + k, {pos, pos + n});
        *off = pos;
        return true;
      }
      if (k < used_.size()) pos = used_[k].second;
    }
    return false;
  }
  void release(int64_t off) {
    for (size_t k = 0; k < used_.size(); ++k)
      if (used_[k].first == off) {
        used_.erase(used_.begin() + k);
        return;
      }
  }
  int64_t cap() const { return cap_; }

 private:
  int64_t cap_;
  std::vector<std::pair<int64_t, int64_t>> used_;
};

}  // namespace

// =========================================================================================
// the batch object
// =========================================================================================
struct sgmev_batch {
  int K = 1;
  int max_slots = 0;
  int num_sms = 152;
  int inner_cap = 1000;  // inner iterations per inner solve
  int outer_cap = 64;
  double eps_inner = 1e-3;

  // pools
  RangeAlloc a_grid, a_data, a_nvec, a_mvec, a_part;
  float2* li = nullptr;
  float4* gq = nullptr;
  float* xh = nullptr;
  float* xl = nullptr;
  float* nh = nullptr;  // N-side FP32 hi/lo (tile-kernel inputs)
  float* nl = nullptr;
  float* mh = nullptr;  // M-side FP32 hi/lo
  float* ml = nullptr;
  float2* part = nullptr;
  // FP64 N-side vectors: b, x, r, d, q, rr, dx
  double* vb = nullptr;
  double* vx = nullptr;
  double* vr = nullptr;
  double* vd = nullptr;
  double* vq = nullptr;
  double* vrr = nullptr;
  double* vdx = nullptr;
  double* dots = nullptr;   // [max_slots * K]
  double* betas = nullptr;  // [max_slots * K]

  // tables
  std::vector<BatchSlot> h_slots;
  std::vector<SlotCtl> h_ctl;
  std::vector<int> h_used;
  BatchSlot* d_slots = nullptr;
  SlotCtl* d_ctl = nullptr;
  ColState* d_col = nullptr;
  SlotCtl* h_ctl_pinned = nullptr;
  // work lists: 0 mult FP32, 1 multT FP32, 2 mult df64, 3 multT df64
  BatchItem* d_items[4] = {nullptr, nullptr, nullptr, nullptr};
  int n_items[4] = {0, 0, 0, 0};
  Seg* d_seg_n = nullptr;
  Seg* d_seg_m = nullptr;
  int n_seg_n = 0, n_seg_m = 0;
  int cap_items = 0, cap_segs = 0;
  int* counters = nullptr;  // 4 launch counters
  bool lists_dirty = true;

  cudaStream_t stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  bool use_graph = true;
  int64_t steps = 0;
  int64_t launches = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

namespace {

void batch_release(sgmev_batch* b) {
  void* ptrs[] = {b->li, b->gq, b->xh, b->xl, b->nh, b->nl, b->mh, b->ml, b->part, b->vb, b->vx,
                  b->vr, b->vd, b->vq, b->vrr, b->vdx, b->dots, b->betas, b->d_slots, b->d_ctl,
                  b->d_col, b->d_items[0], b->d_items[1], b->d_items[2], b->d_items[3],
                  b->d_seg_n, b->d_seg_m, b->counters};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (b->h_ctl_pinned) cudaFreeHost(b->h_ctl_pinned);
  if (b->graph_exec) cudaGraphExecDestroy(b->graph_exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  if (b->stream) cudaStreamDestroy(b->stream);
}

template <typename T>
int balloc(T** p, int64_t count) {
  B_CUDA(cudaMalloc(reinterpret_cast<void**>(p), sizeof(T) * static_cast<size_t>(std::max<int64_t>(count, 1))));
  return SGMEV_OK;
}

// tiling of one slot into the four work-item lists (chunk sizes aim at similar item costs);
// returns the partial-sum elements the slot needs
int64_t plan_slot(const BatchSlot& s, int K, int slot, int64_t target_items,
                  std::vector<BatchItem>* lists, int* nch) {
  int64_t need = 0;
  for (int l = 0; l < 4; ++l) {
    const bool df = l >= 2;
    const bool is_mult = (l % 2) == 0;
    if (is_mult) {
      const int64_t mtiles = s.mpad / (kBB * batch_r(df, K));
      int64_t nsplit = std::max<int64_t>(1, std::min<int64_t>(s.npad / kBGT, cdiv(target_items, mtiles)));
      const int64_t chunk = rup(cdiv(s.npad, nsplit), kBGT);
      nsplit = cdiv(s.npad, chunk);
      nch[l] = static_cast<int>(nsplit);
      for (int64_t q = 0; q < nsplit; ++q)
        for (int64_t t = 0; t < mtiles; ++t)
          lists[l].push_back(BatchItem{slot, static_cast<int>(q), t, q * chunk, std::min(s.npad, (q + 1) * chunk)});
      need = std::max(need, nsplit * s.mpad * K);
    } else {
      const int64_t ntiles = s.npad / (kBB * batch_rg(df, K));
      int64_t nsplit = std::max<int64_t>(1, std::min<int64_t>(s.mpad / kBDT, cdiv(target_items, ntiles)));
      const int64_t chunk = rup(cdiv(s.mpad, nsplit), kBDT);
      nsplit = cdiv(s.mpad, chunk);
      nch[l] = static_cast<int>(nsplit);
      for (int64_t q = 0; q < nsplit; ++q)
        for (int64_t t = 0; t < ntiles; ++t)
          lists[l].push_back(BatchItem{slot, static_cast<int>(q), t, q * chunk, std::min(s.mpad, (q + 1) * chunk)});
      need = std::max(need, nsplit * s.npad * K);
    }
  }
  return need;
}

void drop_graph(sgmev_batch* b) {
  if (b->graph_exec) {
    cudaGraphExecDestroy(b->graph_exec);
    b->graph_exec = nullptr;
  }
  if (b->graph) {
    cudaGraphDestroy(b->graph);
    b->graph = nullptr;
  }
}

int rebuild_lists(sgmev_batch* b) {
  std::vector<BatchItem> lists[4];
  std::vector<Seg> sn, sm;
  for (int s = 0; s < b->max_slots; ++s) {
    if (!b->h_used[s]) continue;
    BatchSlot& sl = b->h_slots[s];
    plan_slot(sl, b->K, s, 2 * b->num_sms, lists, sl.nchunk);
    for (int64_t e = 0; e < sl.npad * b->K; e += kSegLen)
      sn.push_back(Seg{s, sl.nvec_off + e, sl.nvec_off + std::min<int64_t>(sl.npad * b->K, e + kSegLen)});
    for (int64_t e = 0; e < sl.mpad * b->K; e += kSegLen)
      sm.push_back(Seg{s, sl.mvec_off + e, sl.mvec_off + std::min<int64_t>(sl.mpad * b->K, e + kSegLen)});
  }
  size_t need_items = 0;
  for (auto& l : lists) need_items = std::max(need_items, l.size());
  const size_t need_segs = std::max(sn.size(), sm.size());
  if (static_cast<int>(need_items) > b->cap_items) {
    drop_graph(b);
    for (auto& p : b->d_items) {
      cudaFree(p);
      p = nullptr;
    }
    b->cap_items = std::max(static_cast<int>(need_items), 2 * b->cap_items);
    for (auto& p : b->d_items) B_TRY(balloc(&p, b->cap_items));
  }
  if (static_cast<int>(need_segs) > b->cap_segs) {
    drop_graph(b);
    cudaFree(b->d_seg_n);
    cudaFree(b->d_seg_m);
    b->d_seg_n = b->d_seg_m = nullptr;
    b->cap_segs = std::max(static_cast<int>(need_segs), 2 * b->cap_segs);
    B_TRY(balloc(&b->d_seg_n, b->cap_segs));
    B_TRY(balloc(&b->d_seg_m, b->cap_segs));
  }
  bool changed = false;
  for (int l = 0; l < 4; ++l) {
    if (!lists[l].empty())
      B_CUDA(cudaMemcpyAsync(b->d_items[l], lists[l].data(), sizeof(BatchItem) * lists[l].size(), cudaMemcpyHostToDevice, b->stream));
    changed = changed || b->n_items[l] != static_cast<int>(lists[l].size());
    b->n_items[l] = static_cast<int>(lists[l].size());
  }
  if (!sn.empty()) B_CUDA(cudaMemcpyAsync(b->d_seg_n, sn.data(), sizeof(Seg) * sn.size(), cudaMemcpyHostToDevice, b->stream));
  if (!sm.empty()) B_CUDA(cudaMemcpyAsync(b->d_seg_m, sm.data(), sizeof(Seg) * sm.size(), cudaMemcpyHostToDevice, b->stream));
  B_CUDA(cudaMemcpyAsync(b->d_slots, b->h_slots.data(), sizeof(BatchSlot) * b->max_slots, cudaMemcpyHostToDevice, b->stream));
  B_CUDA(cudaStreamSynchronize(b->stream));
  // list lengths are kernel arguments of the captured graph: re-capture when they change
  changed = changed || b->n_seg_n != static_cast<int>(sn.size()) || b->n_seg_m != static_cast<int>(sm.size());
  b->n_seg_n = static_cast<int>(sn.size());
  b->n_seg_m = static_cast<int>(sm.size());
  if (changed) drop_graph(b);
  b->lists_dirty = false;
  return SGMEV_OK;
}

unsigned grid_for(const sgmev_batch* b, int n) {
  return static_cast<unsigned>(std::max(1, std::min(n, 4 * b->num_sms)));
}

// enqueue the launches of one step on b->stream (captured into the graph)
template <int K>
int enqueue_step_k(sgmev_batch* b) {
  const int S = b->max_slots;
  const unsigned tb = 256;
  const unsigned gs = static_cast<unsigned>(cdiv(S, tb));
  const int nn = b->n_seg_n, nm = b->n_seg_m;
  B_CUDA(cudaMemsetAsync(b->counters, 0, sizeof(int) * 4, b->stream));
  // ---- OUTER: r = b - A x with the df64 kernels ----
  b_split_kernel<<<grid_for(b, nn), 256, 0, b->stream>>>(b->d_seg_n, nn, b->d_ctl, PH_OUTER, b->vx, b->nh, b->nl);
  batch_mult_kernel<PolicyDF, K><<<grid_for(b, b->n_items[2]), kBB, 0, b->stream>>>(
      b->d_slots, b->d_ctl, PH_OUTER, b->d_items[2], b->n_items[2], b->counters + 0, b->xh, b->xl, b->li, b->gq, b->nh, b->nl, b->part);
  b_reduce_m_kernel<<<grid_for(b, nm), 256, 0, b->stream>>>(b->d_seg_m, nm, b->d_ctl, PH_OUTER, b->d_slots, K, 2, b->part, b->mh, b->ml);
  batch_multt_kernel<PolicyDF, K><<<grid_for(b, b->n_items[3]), kBB, 0, b->stream>>>(
      b->d_slots, b->d_ctl, PH_OUTER, b->d_items[3], b->n_items[3], b->counters + 1, b->xh, b->xl, b->li, b->gq, b->mh, b->ml, b->part);
  b_reduce_n_kernel<<<grid_for(b, nn), 256, 0, b->stream>>>(b->d_seg_n, nn, b->d_ctl, PH_OUTER, b->d_slots, K, 3, b->part, b->vx, b->vq);
  b_residual_kernel<<<grid_for(b, nn), 256, 0, b->stream>>>(b->d_seg_n, nn, b->d_ctl, b->vb, b->vq, b->vrr);
  b_dot_kernel<K><<<S, 256, 0, b->stream>>>(b->d_slots, b->d_ctl, PH_OUTER, b->vrr, b->vrr, b->dots);
  b_outer_decide_kernel<K><<<gs, tb, 0, b->stream>>>(S, b->d_ctl, b->d_col, b->dots, b->outer_cap);
  b_start_inner_kernel<<<grid_for(b, nn), 256, 0, b->stream>>>(b->d_seg_n, nn, b->d_ctl, b->vrr, b->vdx, b->vr, b->vd);
  // ---- INNER: one CG iteration with FP32 kernels ----
  b_split_kernel<<<grid_for(b, nn), 256, 0, b->stream>>>(b->d_seg_n, nn, b->d_ctl, PH_INNER, b->vd, b->nh, nullptr);
  batch_mult_kernel<PolicyF32, K><<<grid_for(b, b->n_items[0]), kBB, 0, b->stream>>>(
      b->d_slots, b->d_ctl, PH_INNER, b->d_items[0], b->n_items[0], b->counters + 2, b->xh, b->xl, b->li, b->gq, b->nh, b->nl, b->part);
  b_reduce_m_kernel<<<grid_for(b, nm), 256, 0, b->stream>>>(b->d_seg_m, nm, b->d_ctl, PH_INNER, b->d_slots, K, 0, b->part, b->mh, nullptr);
  batch_multt_kernel<PolicyF32, K><<<grid_for(b, b->n_items[1]), kBB, 0, b->stream>>>(
      b->d_slots, b->d_ctl, PH_INNER, b->d_items[1], b->n_items[1], b->counters + 3, b->xh, b->xl, b->li, b->gq, b->mh, b->ml, b->part);
  b_reduce_n_kernel<<<grid_for(b, nn), 256, 0, b->stream>>>(b->d_seg_n, nn, b->d_ctl, PH_INNER, b->d_slots, K, 1, b->part, b->vd, b->vq);
  b_dot_kernel<K><<<S, 256, 0, b->stream>>>(b->d_slots, b->d_ctl, PH_INNER, b->vd, b->vq, b->dots);
  b_inner_alpha_kernel<K><<<static_cast<unsigned>(cdiv(S * K, tb)), tb, 0, b->stream>>>(S, b->d_ctl, b->d_col, b->dots);
  b_inner_update_kernel<K><<<grid_for(b, nn), 256, 0, b->stream>>>(b->d_seg_n, nn, b->d_ctl, b->d_col, b->d_slots, b->vd, b->vq, b->vdx, b->vr);
  b_dot_kernel<K><<<S, 256, 0, b->stream>>>(b->d_slots, b->d_ctl, PH_INNER, b->vr, b->vr, b->dots);
  b_inner_decide_kernel<K><<<gs, tb, 0, b->stream>>>(S, b->d_ctl, b->d_col, b->dots, b->inner_cap, b->betas);
  b_inner_tail_kernel<K><<<grid_for(b, nn), 256, 0, b->stream>>>(b->d_seg_n, nn, b->d_ctl, b->d_slots, b->betas, b->vr, b->vd, b->vdx, b->vx);
  B_CUDA(cudaGetLastError());
  return SGMEV_OK;
}

int enqueue_step(sgmev_batch* b) {
  b->launches += 20;
  return b->K == 16 ? enqueue_step_k<16>(b) : enqueue_step_k<1>(b);
}

int run_step(sgmev_batch* b) {
  if (b->lists_dirty) B_TRY(rebuild_lists(b));
  if (b->use_graph) {
    if (!b->graph_exec) {
      B_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
      const int rc = enqueue_step(b);
      cudaGraph_t g = nullptr;
      const cudaError_t e = cudaStreamEndCapture(b->stream, &g);
      if (rc != SGMEV_OK) {
        if (g) cudaGraphDestroy(g);
        return rc;
      }
      if (e != cudaSuccess) return bfail(SGMEV_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
      b->graph = g;
      B_CUDA(cudaGraphInstantiate(&b->graph_exec, b->graph, 0));
    }
    B_CUDA(cudaGraphLaunch(b->graph_exec, b->stream));
  } else {
    B_TRY(enqueue_step(b));
  }
  b->steps += 1;
  return SGMEV_OK;
}

// stage grid rows (2^l, i) and data into the pools; compute the FP32/df64 forms on the device
__global__ void b_stage_grid_kernel(const double* __restrict__ lp, const double* __restrict__ ix,
                                    int64_t n, int dim, int64_t npad, float2* __restrict__ li,
                                    float4* __restrict__ gq) {
  for (int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; k < npad * dim;
       k += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    double L = 0.0, I = 2.0;
    if (k < n * dim) {
      L = lp[k];
      I = ix[k];
    }
    li[k] = make_float2(static_cast<float>(L), static_cast<float>(I));
    gq[k] = make_float4(static_cast<float>(L), static_cast<float>(1.0 - I), static_cast<float>(1.0 + I), 0.0f);
  }
}

__global__ void b_stage_data_kernel(const double* __restrict__ rows, int64_t m, int dim, int64_t mpad,
                                    float* __restrict__ xh, float* __restrict__ xl) {
  for (int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; k < mpad * dim;
       k += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int t = static_cast<int>(k / mpad);
    const int64_t j = k - static_cast<int64_t>(t) * mpad;
    const double x = j < m ? rows[j * dim + t] : 0.0;
    const float h = static_cast<float>(x);
    xh[k] = h;
    xl[k] = static_cast<float>(x - static_cast<double>(h));
  }
}

// y [m x K] row-major doubles -> M-side hi/lo pools (padding 0)
__global__ void b_stage_y_kernel(const double* __restrict__ y, int64_t m, int64_t mpad, int K,
                                 float* __restrict__ vh, float* __restrict__ vl) {
  for (int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; k < mpad * K;
       k += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const double v = (k / K) < m ? y[k] : 0.0;
    const float h = static_cast<float>(v);
    vh[k] = h;
    vl[k] = static_cast<float>(v - static_cast<double>(h));
  }
}

}  // namespace

// =========================================================================================
// C ABI
// =========================================================================================
extern "C" {

SGMEV_API int sgmev_batch_create(sgmev_batch** out, int max_slots, int rhs, int64_t grid_capacity,
                                 int64_t data_capacity, const char* params_json) {
  using namespace sgmev;
  if (!out) return bfail(SGMEV_ERR_INVALID, "out is NULL");
  *out = nullptr;
  if (max_slots < 1 || max_slots > 4096) return bfail(SGMEV_ERR_INVALID, "max_slots must be in [1, 4096]");
  if (rhs != 1 && rhs != 16) return bfail(SGMEV_ERR_INVALID, "rhs must be 1 or 16");
  if (grid_capacity < 1 || data_capacity < 1) return bfail(SGMEV_ERR_INVALID, "capacities must be >= 1");
  (void)params_json;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return bfail(SGMEV_ERR_NO_DEVICE, "no CUDA device is visible");
  }
  sgmev_batch* b = new sgmev_batch;
  b->K = rhs;
  b->max_slots = max_slots;
  auto bail = [&](int rc) {
    batch_release(b);
    delete b;
    return rc;
  };
#define C_TRY(expr)                 \
  do {                              \
    int rc_ = (expr);               \
    if (rc_ != SGMEV_OK) return bail(rc_); \
  } while (0)
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&b->num_sms, cudaDevAttrMultiProcessorCount, dev);
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(bfail(SGMEV_ERR_CUDA, "cudaStreamCreate"));
  cudaEventCreate(&b->ev0);
  cudaEventCreate(&b->ev1);
  // pool capacities (elements). Grid: padded rows x dim; data: dim x padded points.
  const int64_t gcap = grid_capacity + 16 * 512 * static_cast<int64_t>(max_slots);
  const int64_t dcap = data_capacity + 16 * 1024 * static_cast<int64_t>(max_slots);
  b->a_grid = RangeAlloc(gcap);
  b->a_data = RangeAlloc(dcap);
  const int64_t ncap = (gcap)*rhs;  // N-side vectors (npad * K) <= grid rows * K
  const int64_t mcap = (dcap)*rhs;
  b->a_nvec = RangeAlloc(ncap);
  b->a_mvec = RangeAlloc(mcap);
  const int64_t pcap = 8 * std::max(ncap, mcap) + 2 * static_cast<int64_t>(b->num_sms) * 512 * rhs;
  b->a_part = RangeAlloc(pcap);
  C_TRY(balloc(&b->li, gcap));
  C_TRY(balloc(&b->gq, gcap));
  C_TRY(balloc(&b->xh, dcap));
  C_TRY(balloc(&b->xl, dcap));
  C_TRY(balloc(&b->nh, ncap));
  C_TRY(balloc(&b->nl, ncap));
  C_TRY(balloc(&b->mh, mcap));
  C_TRY(balloc(&b->ml, mcap));
  C_TRY(balloc(&b->part, pcap));
  C_TRY(balloc(&b->vb, ncap));
  C_TRY(balloc(&b->vx, ncap));
  C_TRY(balloc(&b->vr, ncap));
  C_TRY(balloc(&b->vd, ncap));
  C_TRY(balloc(&b->vq, ncap));
  C_TRY(balloc(&b->vrr, ncap));
  C_TRY(balloc(&b->vdx, ncap));
  C_TRY(balloc(&b->dots, static_cast<int64_t>(max_slots) * rhs));
  C_TRY(balloc(&b->betas, static_cast<int64_t>(max_slots) * rhs));
  C_TRY(balloc(&b->d_slots, max_slots));
  C_TRY(balloc(&b->d_ctl, max_slots));
  C_TRY(balloc(&b->d_col, static_cast<int64_t>(max_slots) * rhs));
  C_TRY(balloc(&b->counters, 4));
  if (cudaMallocHost(&b->h_ctl_pinned, sizeof(SlotCtl) * max_slots) != cudaSuccess)
    return bail(bfail(SGMEV_ERR_OOM, "cudaMallocHost"));
  b->h_slots.assign(max_slots, BatchSlot{});
  b->h_ctl.assign(max_slots, SlotCtl{});
  b->h_used.assign(max_slots, 0);
  if (cudaMemset(b->d_ctl, 0, sizeof(SlotCtl) * max_slots) != cudaSuccess ||
      cudaMemset(b->d_slots, 0, sizeof(BatchSlot) * max_slots) != cudaSuccess)
    return bail(bfail(SGMEV_ERR_CUDA, "cudaMemset"));
#undef C_TRY
  *out = b;
  return SGMEV_OK;
}

SGMEV_API int sgmev_batch_destroy(sgmev_batch* b) {
  if (!b) return SGMEV_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  batch_release(b);
  delete b;
  return SGMEV_OK;
}

SGMEV_API int sgmev_batch_footprint(int dim, int64_t n_grid, int64_t n_data, int rhs,
                                    int64_t* grid_elems, int64_t* data_elems) {
  if (dim < 1 || dim > kMaxBatchDim || n_grid < 1 || n_data < 0 || (rhs != 1 && rhs != 16))
    return bfail(SGMEV_ERR_INVALID, "bad problem size");
  const int64_t npad = rup(n_grid, 512);
  const int64_t mpad = std::max<int64_t>(rup(std::max<int64_t>(n_data, 1), 1024), 1024);
  if (grid_elems) *grid_elems = npad * dim;
  if (data_elems) *data_elems = mpad * dim;
  return SGMEV_OK;
}

SGMEV_API int sgmev_batch_add(sgmev_batch* b, int dim, int64_t n_grid, const double* level_pow2,
                              const double* index, int64_t n_data, const double* data,
                              const double* y, double lambda, double epsilon,
                              int64_t max_iterations, int* slot_out) {
  using namespace sgmev;
  if (!b || !slot_out) return bfail(SGMEV_ERR_INVALID, "NULL argument");
  *slot_out = -1;
  if (dim < 1 || dim > kMaxBatchDim) return bfail(SGMEV_ERR_UNSUPPORTED, "batch problems need 1 <= dim <= 16");
  if (n_grid < 1 || n_data < 1 || !level_pow2 || !index || !data || !y)
    return bfail(SGMEV_ERR_INVALID, "empty problem or NULL pointer");
  if (!(epsilon > 0.0) || max_iterations < 1 || !(lambda >= 0.0))
    return bfail(SGMEV_ERR_INVALID, "bad epsilon / max_iterations / lambda");
  for (int64_t k = 0; k < n_grid * dim; ++k) {
    const double L = level_pow2[k], I = index[k];
    if (!(L >= 2.0) || L > 16777216.0 || std::floor(std::log2(L)) != std::log2(L) || !(I >= 1.0) ||
        !(I < L) || std::fmod(I, 2.0) != 1.0)
      return bfail(SGMEV_ERR_UNSUPPORTED, "grid entry " + std::to_string(k) + " is not a hat (2^l, odd i)");
  }
  int slot = -1;
  for (int s = 0; s < b->max_slots; ++s)
    if (!b->h_used[s]) {
      slot = s;
      break;
    }
  if (slot < 0) return bfail(SGMEV_ERR_OOM, "no free slot");
  BatchSlot sl{};
  sl.dim = dim;
  sl.active = 1;
  sl.n = n_grid;
  sl.npad = rup(n_grid, 512);
  sl.m = n_data;
  sl.mpad = rup(n_data, 1024);
  const int K = b->K;
  int64_t goff, doff, noff, moff, poff;
  // partial capacity: the largest chunk count of the four plans times its stride
  std::vector<BatchItem> plan_lists[4];
  const int64_t pneed = plan_slot(sl, K, 0, 2 * b->num_sms, plan_lists, sl.nchunk);
  if (!b->a_grid.alloc(sl.npad * dim, &goff)) return bfail(SGMEV_ERR_OOM, "grid pool full");
  if (!b->a_data.alloc(sl.mpad * dim, &doff)) {
    b->a_grid.release(goff);
    return bfail(SGMEV_ERR_OOM, "data pool full");
  }
  if (!b->a_nvec.alloc(sl.npad * K, &noff)) {
    b->a_grid.release(goff);
    b->a_data.release(doff);
    return bfail(SGMEV_ERR_OOM, "vector pool full");
  }
  if (!b->a_mvec.alloc(sl.mpad * K, &moff)) {
    b->a_grid.release(goff);
    b->a_data.release(doff);
    b->a_nvec.release(noff);
    return bfail(SGMEV_ERR_OOM, "data-vector pool full");
  }
  if (!b->a_part.alloc(pneed, &poff)) {
    b->a_grid.release(goff);
    b->a_data.release(doff);
    b->a_nvec.release(noff);
    b->a_mvec.release(moff);
    return bfail(SGMEV_ERR_OOM, "partial-sum pool full");
  }
  sl.grid_off = goff;
  sl.data_off = doff;
  sl.nvec_off = noff;
  sl.mvec_off = moff;
  sl.part_off = poff;
  // stage inputs (temporary device copies)
  double *d_l = nullptr, *d_i = nullptr, *d_x = nullptr, *d_y = nullptr;
  auto cleanup = [&]() {
    cudaFree(d_l);
    cudaFree(d_i);
    cudaFree(d_x);
    cudaFree(d_y);
  };
  auto undo = [&](int rc) {
    cleanup();
    b->a_grid.release(goff);
    b->a_data.release(doff);
    b->a_nvec.release(noff);
    b->a_mvec.release(moff);
    b->a_part.release(poff);
    return rc;
  };
  if (cudaMalloc(&d_l, sizeof(double) * n_grid * dim) != cudaSuccess ||
      cudaMalloc(&d_i, sizeof(double) * n_grid * dim) != cudaSuccess ||
      cudaMalloc(&d_x, sizeof(double) * n_data * dim) != cudaSuccess ||
      cudaMalloc(&d_y, sizeof(double) * n_data * K) != cudaSuccess)
    return undo(bfail(SGMEV_ERR_OOM, "staging allocation"));
  cudaMemcpyAsync(d_l, level_pow2, sizeof(double) * n_grid * dim, cudaMemcpyHostToDevice, b->stream);
  cudaMemcpyAsync(d_i, index, sizeof(double) * n_grid * dim, cudaMemcpyHostToDevice, b->stream);
  cudaMemcpyAsync(d_x, data, sizeof(double) * n_data * dim, cudaMemcpyHostToDevice, b->stream);
  cudaMemcpyAsync(d_y, y, sizeof(double) * n_data * K, cudaMemcpyHostToDevice, b->stream);
  const unsigned gb = 1216;
  b_stage_grid_kernel<<<gb, 256, 0, b->stream>>>(d_l, d_i, n_grid, dim, sl.npad, b->li + goff, b->gq + goff);
  b_stage_data_kernel<<<gb, 256, 0, b->stream>>>(d_x, n_data, dim, sl.mpad, b->xh + doff, b->xl + doff);
  b_stage_y_kernel<<<gb, 256, 0, b->stream>>>(d_y, n_data, sl.mpad, K, b->mh + moff, b->ml + moff);
  cudaMemsetAsync(b->vx + noff, 0, sizeof(double) * sl.npad * K, b->stream);
  cudaError_t e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) return undo(bfail(SGMEV_ERR_CUDA, std::string("stage: ") + cudaGetErrorString(e)));
  // b = B^T y with the df64 kernels: one multT launch over this slot alone
  b->h_slots[slot] = sl;
  b->h_used[slot] = 1;
  {
    std::vector<BatchItem> it = plan_lists[3];  // multT df64 items of this slot
    for (auto& item : it) item.slot = slot;
    BatchItem* d_it = nullptr;
    Seg* d_sg = nullptr;
    std::vector<Seg> sn;
    for (int64_t q = 0; q < sl.npad * K; q += kSegLen)
      sn.push_back(Seg{slot, noff + q, noff + std::min<int64_t>(sl.npad * K, q + kSegLen)});
    if (cudaMalloc(&d_it, sizeof(BatchItem) * it.size()) != cudaSuccess ||
        cudaMalloc(&d_sg, sizeof(Seg) * sn.size()) != cudaSuccess) {
      cudaFree(d_it);
      b->h_used[slot] = 0;
      return undo(bfail(SGMEV_ERR_OOM, "staging allocation"));
    }
    SlotCtl c{};
    c.phase = PH_OUTER;
    c.eps = epsilon;
    c.eps_inner = b->eps_inner;
    c.max_it = static_cast<int>(std::min<int64_t>(max_iterations, 1 << 30));
    c.lm = lambda * static_cast<double>(n_data);
    b->h_ctl[slot] = c;
    cudaMemcpyAsync(b->d_slots + slot, &b->h_slots[slot], sizeof(BatchSlot), cudaMemcpyHostToDevice, b->stream);
    cudaMemcpyAsync(b->d_ctl + slot, &c, sizeof(SlotCtl), cudaMemcpyHostToDevice, b->stream);
    cudaMemcpyAsync(d_it, it.data(), sizeof(BatchItem) * it.size(), cudaMemcpyHostToDevice, b->stream);
    cudaMemcpyAsync(d_sg, sn.data(), sizeof(Seg) * sn.size(), cudaMemcpyHostToDevice, b->stream);
    cudaMemsetAsync(b->counters, 0, sizeof(int) * 4, b->stream);
    if (K == 16)
      batch_multt_kernel<PolicyDF, 16><<<grid_for(b, static_cast<int>(it.size())), kBB, 0, b->stream>>>(
          b->d_slots, b->d_ctl, PH_OUTER, d_it, static_cast<int>(it.size()), b->counters, b->xh, b->xl, b->li, b->gq, b->mh, b->ml, b->part);
    else
      batch_multt_kernel<PolicyDF, 1><<<grid_for(b, static_cast<int>(it.size())), kBB, 0, b->stream>>>(
          b->d_slots, b->d_ctl, PH_OUTER, d_it, static_cast<int>(it.size()), b->counters, b->xh, b->xl, b->li, b->gq, b->mh, b->ml, b->part);
    b_reduce_n_kernel<<<grid_for(b, static_cast<int>(sn.size())), 256, 0, b->stream>>>(d_sg, static_cast<int>(sn.size()), b->d_ctl, PH_OUTER, b->d_slots, K, 3, b->part, nullptr, b->vb);
    e = cudaStreamSynchronize(b->stream);
    cudaFree(d_it);
    cudaFree(d_sg);
    if (e != cudaSuccess) {
      b->h_used[slot] = 0;
      return undo(bfail(SGMEV_ERR_CUDA, std::string("b = B^T y: ") + cudaGetErrorString(e)));
    }
  }
  cleanup();
  b->lists_dirty = true;
  *slot_out = slot;
  return SGMEV_OK;
}

SGMEV_API int sgmev_batch_remove(sgmev_batch* b, int slot) {
  if (!b || slot < 0 || slot >= b->max_slots || !b->h_used[slot])
    return bfail(SGMEV_ERR_INVALID, "no such slot");
  B_CUDA(cudaStreamSynchronize(b->stream));
  const BatchSlot& sl = b->h_slots[slot];
  b->a_grid.release(sl.grid_off);
  b->a_data.release(sl.data_off);
  b->a_nvec.release(sl.nvec_off);
  b->a_mvec.release(sl.mvec_off);
  b->a_part.release(sl.part_off);
  b->h_used[slot] = 0;
  b->h_slots[slot] = BatchSlot{};
  SlotCtl c{};
  c.phase = PH_EMPTY;
  B_CUDA(cudaMemcpyAsync(b->d_ctl + slot, &c, sizeof(SlotCtl), cudaMemcpyHostToDevice, b->stream));
  B_CUDA(cudaStreamSynchronize(b->stream));
  b->lists_dirty = true;
  return SGMEV_OK;
}

// Advance every unfinished problem by `steps` steps (one inner CG iteration or one outer residual
// each); then report each slot's phase (0 empty, 1/2 running, 3 done) in phases[max_slots].
SGMEV_API int sgmev_batch_step(sgmev_batch* b, int steps, int* phases) {
  if (!b || steps < 0) return bfail(SGMEV_ERR_INVALID, "bad arguments");
  for (int k = 0; k < steps; ++k) B_TRY(run_step(b));
  B_CUDA(cudaMemcpyAsync(b->h_ctl_pinned, b->d_ctl, sizeof(SlotCtl) * b->max_slots, cudaMemcpyDeviceToHost, b->stream));
  B_CUDA(cudaStreamSynchronize(b->stream));
  if (phases)
    for (int s = 0; s < b->max_slots; ++s) phases[s] = b->h_used[s] ? b->h_ctl_pinned[s].phase : PH_EMPTY;
  return SGMEV_OK;
}

// Run until every problem in the batch is done (or max_steps steps); returns the steps taken.
SGMEV_API int sgmev_batch_solve(sgmev_batch* b, int64_t max_steps, int64_t* steps_taken) {
  if (!b) return bfail(SGMEV_ERR_INVALID, "NULL batch");
  std::vector<int> ph(b->max_slots);
  int64_t k = 0;
  for (; k < max_steps; ++k) {
    B_TRY(sgmev_batch_step(b, 1, ph.data()));
    bool running = false;
    for (int s = 0; s < b->max_slots; ++s) running = running || ph[s] == PH_OUTER || ph[s] == PH_INNER;
    if (!running) {
      ++k;
      break;
    }
  }
  if (steps_taken) *steps_taken = k;
  return SGMEV_OK;
}

// alpha [n_grid x K] row-major; iterations: inner CG iterations; residual: max over columns of
// ||b - A alpha||^2 / ||b - A alpha_0||^2 at the last outer step; phase: the slot's phase.
SGMEV_API int sgmev_batch_result(sgmev_batch* b, int slot, double* alpha, int64_t* iterations,
                                 double* residual, int* phase) {
  if (!b || slot < 0 || slot >= b->max_slots || !b->h_used[slot])
    return bfail(SGMEV_ERR_INVALID, "no such slot");
  const BatchSlot& sl = b->h_slots[slot];
  const int K = b->K;
  SlotCtl c{};
  std::vector<ColState> cs(K);
  B_CUDA(cudaMemcpyAsync(&c, b->d_ctl + slot, sizeof(SlotCtl), cudaMemcpyDeviceToHost, b->stream));
  B_CUDA(cudaMemcpyAsync(cs.data(), b->d_col + static_cast<int64_t>(slot) * K, sizeof(ColState) * K, cudaMemcpyDeviceToHost, b->stream));
  if (alpha) B_CUDA(cudaMemcpyAsync(alpha, b->vx + sl.nvec_off, sizeof(double) * sl.n * K, cudaMemcpyDeviceToHost, b->stream));
  B_CUDA(cudaStreamSynchronize(b->stream));
  if (iterations) *iterations = c.total_it;
  if (residual) {
    double worst = 0.0;
    for (int k = 0; k < K; ++k) worst = std::max(worst, cs[k].r0 > 0.0 ? cs[k].rnorm2 / cs[k].r0 : 0.0);
    *residual = worst;
  }
  if (phase) *phase = c.phase;
  return SGMEV_OK;
}

SGMEV_API int sgmev_batch_info(sgmev_batch* b, int64_t* steps, int64_t* launches,
                               int* free_slots) {
  if (!b) return bfail(SGMEV_ERR_INVALID, "NULL batch");
  if (steps) *steps = b->steps;
  if (launches) *launches = b->launches;
  if (free_slots) {
    int f = 0;
    for (int s = 0; s < b->max_slots; ++s) f += b->h_used[s] ? 0 : 1;
    *free_slots = f;
  }
  return SGMEV_OK;
}

}  // extern "C"
