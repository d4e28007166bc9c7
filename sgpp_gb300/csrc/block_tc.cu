// Products with 16 right-hand sides on the tensor cores: FP16 or BF16 tcgen05 MMAs over weighted
// one-hot tiles of the materialised subspace products (the scheme is described in block_tc.h).
//
// Both kernels run one CTA per SM: producer teams of four warps (three teams by default), one MMA
// warp and one loader warp.
//   producers  read the packed FP16 / BF16 products (2 bytes + the cell index per point and
//              subspace, one 32-bit word) of a tile of 128 points and a group of 16 chunks and
//              write the tile's rows of E into a stage (shared or tensor memory): 16 bytes per
//              point and chunk, one non-zero per point and subspace (thread = point);
//   MMA warp   one thread waits for a full stage and issues its eight 128 x 32 x 16 MMAs, then
//              commits them to the stage's "empty" barrier, which frees the stage for the
//              producers once the tensor cores have read it.
// A stage holds 128 points x 16 chunks in the canonical no-swizzle layout: the 16-byte chunk of
// point p and chunk q at (p / 8) * 2048 + q * 128 + (p % 8) * 16. Read K-major it is the A
// operand of mult (M = points, K = rows); read MN-major it is the A operand of multT (M = rows,
// K = points). Every wait is bounded: a wait that runs out sets the status word and the CTA
// finishes without further work, after its issued MMAs have completed and its tensor memory is
// freed.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "block_tc.h"
#include "devmem.h"
#include "tc_ptx.cuh"

namespace sgmev {
namespace {

// The producers form teams of 4 warps (one warp per 32 points of a stage, the tensor-memory lanes
// its warp may access); team t writes stages t, t + teams, t + 2 teams, ... so that the teams'
// waits and latencies overlap. Behind the producers: the MMA warp and the loader warp.
// Ring safety: a parity wait tells a barrier's phase only from the one before it, so no waiter may
// run two phases ahead. Load buffer b serves stages b, b + loads, ...; with loads a multiple of
// teams they all belong to one team, which waits for each in turn (bulk copies may land out of
// order, so a buffer shared between teams could be waited on for its next use before its current
// one had landed). An E stage slot may pass between teams: its waits stay within one phase when
// teams <= stages, since a team's previous stage already waited for the MMAs of the stage before.
constexpr int kTeamWarps = 4;
constexpr int kMaxTeams = 4;
constexpr int kMaxThreads = (kTeamWarps * kMaxTeams + 2) * 32;
constexpr uint32_t kStageBytes = 128u * 16u * 16u;  // 128 points x 16 chunks x 16 bytes
constexpr uint32_t kCoefBytes = 4096u * 2u;         // 128 rows x 32 columns of 16-bit values
constexpr uint32_t kQBytes = 4096u * 2u;            // 128 points x 32 columns of 16-bit values
constexpr uint32_t kSlotRow = 128u * 4u;            // one slot's packed words of a tile
constexpr uint32_t kHeaderAt = 16u * kSlotRow;      // a group has at most 16 slots, then its
constexpr uint32_t kLoadBytes = kHeaderAt + 128u;   // 128-byte chunk header
constexpr int32_t kUnusedBase = 0x40000000;         // shift base of a chunk no slot uses
constexpr uint64_t kWaitNs = 2000000000ull;         // a bounded wait gives up after 2 s
constexpr int kMaxStages = 6;
constexpr int kMaxLoads = 12;
constexpr int kMaxWindow = 3;  // stages the MMA thread interleaves
// core-matrix strides of the operands: 128 bytes between neighbouring core matrices along the
// row dimension of a chunk / K-step (8 elements), 2048 bytes between groups of 8 points or of 8
// output columns
constexpr uint32_t kCoreK = 128, kCoreMN = 2048;
// operand A of multT (E^T, MN-major): core-matrix offsets along the points (K, leading) and along
// the rows (M, strided)
constexpr uint32_t kMnA_LBO = 2048, kMnA_SBO = 128;

__host__ __device__ inline int64_t cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Position in a ring of buffers: the buffer index and the number of completed rounds, whose
// parity is the phase to wait for. Advanced without divisions: a 64-bit division is a software
// routine on the GPU, and four of them per stage had cost more than the stage's own work.
struct Ring {
  int idx = 0;
  uint32_t round = 0;
  __device__ __forceinline__ void next(int n) {
    if (++idx == n) {
      idx = 0;
      ++round;
    }
  }
  // `by` positions on (by <= n): a team's next stage
  __device__ __forceinline__ void step(int by, int n) {
    idx += by;
    if (idx >= n) {
      idx -= n;
      ++round;
    }
  }
};

// barrier and bookkeeping words behind the buffers
struct Sync {
  uint64_t full[kMaxStages];   // E stage written (producers)
  uint64_t empty[kMaxStages];  // E stage read by the tensor cores (MMA commit)
  uint64_t lfull[kMaxLoads];   // packed products of a stage arrived (bulk copies)
  uint64_t lempty[kMaxLoads];  // packed products read (producers)
  uint64_t qfull[2];           // Q tile arrived (multT)
  uint64_t qempty[2];          // Q tile read by the tensor cores (multT)
  uint64_t cfull;              // coefficient rows of a pass arrived (mult)
  uint64_t pass;               // MMAs of a pass completed (mult)
  uint64_t last;
  uint32_t tmem;
  volatile int abort;
};

__device__ __forceinline__ void fail_wait(Sync* sy, int* status, int code) {
  sy->abort = 1;
  atomicOr(status, code);
}

// The MMA warp's decisions are warp-uniform (its lanes run one loop together): a bounded wait
// that every lane passed, and the abort flag as lane 0 read it.
__device__ __forceinline__ bool warp_wait(uint32_t mbar, uint32_t parity) {
  return __all_sync(0xffffffffu, tc::mbar_wait_ns(mbar, parity, kWaitNs));
}
__device__ __forceinline__ bool warp_aborted(const Sync* sy) {
  return __shfl_sync(0xffffffffu, sy->abort, 0) != 0;
}

// BF16 high/low split: v = hi + lo to about 16 significant bits
__device__ __forceinline__ void split_bf16(float v, uint16_t* hi, uint16_t* lo) {
  const __nv_bfloat16 h = __float2bfloat16_rn(v);
  const __nv_bfloat16 l = __float2bfloat16_rn(v - __bfloat162float(h));
  *hi = *reinterpret_cast<const uint16_t*>(&h);
  *lo = *reinterpret_cast<const uint16_t*>(&l);
}

// FP16 high/low split: v = hi + lo to about 22 significant bits (v already scaled into FP16's range)
__device__ __forceinline__ void split_f16(float v, uint16_t* hi, uint16_t* lo) {
  const __half h = __float2half_rn(v);
  const __half l = __float2half_rn(v - __half2float(h));
  *hi = *reinterpret_cast<const uint16_t*>(&h);
  *lo = *reinterpret_cast<const uint16_t*>(&l);
}

template <bool F16>
__device__ __forceinline__ void split_pair(float v, uint16_t* hi, uint16_t* lo) {
  if constexpr (F16)
    split_f16(v, hi, lo);
  else
    split_bf16(v, hi, lo);
}

// byte offset of element (column n, row r) of a 32-column operand block in the K-major layout
__host__ __device__ inline uint32_t opnd_off(int n, int r) {
  return static_cast<uint32_t>((n >> 3) * 2048 + (r >> 3) * 128 + (n & 7) * 16 + (r & 7) * 2);
}

// ---- bulk copies (the loader thread) ------------------------------------------------------------
__device__ __forceinline__ void bulk_expect(uint32_t mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes)
               : "memory");
}
// global -> shared, `bytes` a multiple of 16, both addresses 16-byte aligned
__device__ __forceinline__ void bulk_copy(uint32_t dst, const void* src, uint32_t bytes,
                                          uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          dst),
      "l"(src), "r"(bytes), "r"(mbar)
      : "memory");
}

// The packed products of stage (tile, group) into load buffer `buf`. They are stored tile by
// tile, pc[tile][slot][128 points], so a group's slots of a tile are one contiguous run and a stage
// is one bulk copy (one 512-byte copy per slot kept the copy engine, not the memory, busy).
// The group's chunk header comes along into the same buffer (a header read from global memory
// per stage, on the producers' critical path, cost them more than writing the stage).
// gs: the group's first slot and slot count.
__device__ __forceinline__ void load_stage(unsigned char* buf, uint32_t mbar,
                                           const uint32_t* __restrict__ pc, int2 gs,
                                           const BlockHeader* __restrict__ gheader, int n_slots,
                                           int group, int64_t tile) {
  const uint32_t bytes = static_cast<uint32_t>(gs.y) * kSlotRow;
  bulk_expect(mbar, bytes + static_cast<uint32_t>(sizeof(BlockHeader)));
  bulk_copy(tc::smem_u32(buf), pc + (tile * n_slots + gs.x) * 128, bytes, mbar);
  bulk_copy(tc::smem_u32(buf + kHeaderAt), gheader + group, sizeof(BlockHeader), mbar);
}

// ---- producer: one stage of E ----------------------------------------------------------------
// A packed word holds a point's 16-bit product in one subspace (low half) and 16 x its cell c in
// that subspace (high half). Each group carries a header (BlockHeader): for chunk q, the byte
// offset of its slot's row in the load buffer and the shift base 128 x (which of the slot's
// chunks q is), or kUnusedBase for a chunk no slot uses. The chunk holds the point's product at
// element c - 8 x that index when that lies in 0..7, zeros otherwise; with s = 16 c - base, word k
// of the chunk (elements 2k, 2k + 1) is the product shifted left by s - 32 k, since a shift by 32
// or more, or by a negative amount read as unsigned, gives 0. Thread p of a team writes the 16
// chunks of point p.
struct ChunkWords {
  uint32_t v[16];  // product bits
  uint32_t s[16];  // shift of the product within the chunk's 128 bits
};

__device__ __forceinline__ uint32_t shl_clamped(uint32_t v, uint32_t s) {
  uint32_t r;
  asm("shl.b32 %0, %1, %2;" : "=r"(r) : "r"(v), "r"(s));
  return r;
}

__device__ __forceinline__ void read_chunks(ChunkWords& C, const unsigned char* lbuf, int p) {
  const BlockHeader& hd = *reinterpret_cast<const BlockHeader*>(lbuf + kHeaderAt);
  int32_t row[16], base[16];
#pragma unroll
  for (int i = 0; i < 16; i += 4) {
    const int4 r4 = *reinterpret_cast<const int4*>(&hd.row[i]);
    const int4 b4 = *reinterpret_cast<const int4*>(&hd.base[i]);
    row[i] = r4.x, row[i + 1] = r4.y, row[i + 2] = r4.z, row[i + 3] = r4.w;
    base[i] = b4.x, base[i + 1] = b4.y, base[i + 2] = b4.z, base[i + 3] = b4.w;
  }
  const unsigned char* lp = lbuf + 4 * p;
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    const uint32_t w = *reinterpret_cast<const uint32_t*>(lp + row[i]);
    C.v[i] = w & 0xFFFFu;
    C.s[i] = (w >> 16) - static_cast<uint32_t>(base[i]);
  }
}

// words 4i .. 4i + 3 of a point's row of E: chunk i
__device__ __forceinline__ void chunk_words(const ChunkWords& C, int i, uint32_t& r0, uint32_t& r1,
                                            uint32_t& r2, uint32_t& r3) {
  r0 = shl_clamped(C.v[i], C.s[i]);
  r1 = shl_clamped(C.v[i], C.s[i] - 32u);
  r2 = shl_clamped(C.v[i], C.s[i] - 64u);
  r3 = shl_clamped(C.v[i], C.s[i] - 96u);
}

__device__ __forceinline__ void write_chunks(unsigned char* stage, int p, const ChunkWords& C) {
  unsigned char* base = stage + (p >> 3) * 2048 + (p & 7) * 16;
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    uint4 q;
    chunk_words(C, i, q.x, q.y, q.z, q.w);
    *reinterpret_cast<uint4*>(base + i * 128) = q;
  }
}

// The loader warp's copy of gslots for a window of 32 groups, one per lane: a global load of the
// group's slots per stage, waited for before each copy could be issued, had set the pace of the
// whole pipeline. The group index is warp-uniform.
struct GroupSlots {
  int2 lane_gs = make_int2(0, 0);
  int window = -1;
  __device__ __forceinline__ int2 get(const int2* __restrict__ gslots, int n_groups, int group) {
    const int w0 = group & ~31;
    if (w0 != window) {
      window = w0;
      const int g = w0 + static_cast<int>(threadIdx.x & 31);
      lane_gs = g < n_groups ? __ldg(gslots + g) : make_int2(0, 0);
    }
    return make_int2(__shfl_sync(0xffffffffu, lane_gs.x, group & 31),
                     __shfl_sync(0xffffffffu, lane_gs.y, group & 31));
  }
};

// Where a kernel's stages come from: stage k of the kernel's order is (major, minor) =
// (k / n_minor, k % n_minor), in the mult (group, tile of the CTA) and in the multT (tile of the
// stream, group of the pass).
struct StageSource {
  const uint32_t* __restrict__ pc;
  const int2* __restrict__ gslots;
  const BlockHeader* __restrict__ gheader;
  int n_slots, n_groups, n_minor;
  int group0;        // multT: first group of the pass
  int64_t tile0;     // first tile of the CTA (mult) or of the stream (multT)
  bool tiles_minor;  // the mult's order
  int64_t total;     // stages of the CTA
};

// The copies of one team's stages, issued by the team's first warp: the team's first
// loads / teams stages up front, then stage k + loads into the buffer of stage k as soon as the
// team's four warps have read stage k. A team's load buffers are its own, so no other warp takes
// part (one loader warp issuing every stage's copy after a hand-off per stage had been the
// slowest link of the pipeline).
struct TeamLoads {
  int64_t k = 0;  // next stage to load
  int major = 0, minor = 0;
  Ring ring;      // its buffer
  GroupSlots gsl;
  __device__ __forceinline__ void init(int team, int n_minor) {
    k = team;
    major = team / n_minor;
    minor = team % n_minor;
    ring = Ring{team, 0u};
  }
  __device__ __forceinline__ void step(int teams, int n_minor, int loads) {
    k += teams;
    minor += teams;
    while (minor >= n_minor) {
      minor -= n_minor;
      ++major;
    }
    ring.step(teams, loads);
  }
  // by the whole warp; the elected lane issues
  __device__ __forceinline__ void issue(Sync* sy, unsigned char* lb, const StageSource& src) {
    const int group = src.tiles_minor ? major : src.group0 + minor;
    const int64_t tile = src.tile0 + (src.tiles_minor ? minor : major);
    const int2 gs = gsl.get(src.gslots, src.n_groups, group);
    if (tc::elect_one()) {
      tc::fence_proxy_async();  // the team's reads of the buffer come before the copy's writes
      load_stage(lb + static_cast<size_t>(ring.idx) * kLoadBytes,
                 tc::smem_u32(&sy->lfull[ring.idx]), src.pc, gs, src.gheader, src.n_slots, group,
                 tile);
    }
    __syncwarp();
  }
  // before the CTA exits: the last copy into each of the team's buffers has landed (the copies
  // of an aborted run must not write shared memory after the CTA is gone)
  __device__ __forceinline__ void drain(Sync* sy, int* status, int teams, int loads, int team) {
    for (int64_t j = k - teams; j >= team && j >= k - loads; j -= teams) {
      const int b = static_cast<int>(j % loads);
      if (!warp_wait(tc::smem_u32(&sy->lfull[b]), static_cast<uint32_t>((j / loads) & 1)) &&
          (threadIdx.x & 31) == 0)
        atomicOr(status, 128);
    }
  }
};

// A team's part of its next stage: wait for the packed products, read them, free the load
// buffer (the team's first warp then loads the team's stage `loads` ahead into it), wait for the
// E stage to be free, write it, mark it full, step both rings past the other teams' stages.
// TMEM: the stage's rows go to tensor memory (lane = point, 4 columns per chunk: the chunk's 8
// 16-bit elements as 4 pairs) with two 32-column stores per thread instead of shared memory, so the
// tensor cores read A without the shared-memory traffic of writing and reading it.
// False when a wait ran out.
template <bool TMEM>
__device__ __forceinline__ bool produce(Sync* sy, int* status, unsigned char* st,
                                        unsigned char* lb, Ring& lr, int loads, Ring& sr,
                                        int stages, uint32_t a_taddr, int p, int teams,
                                        TeamLoads& tl, const StageSource& src, bool issuer) {
  const int b = lr.idx;
  // the warp's lanes decide together (a lane that gave up alone would leave the others waiting
  // at the warp's synchronisation below)
  if (!__all_sync(0xffffffffu, tc::mbar_wait_ns(tc::smem_u32(&sy->lfull[b]), lr.round & 1u,
                                                kWaitNs))) {
    fail_wait(sy, status, 32);
    return false;
  }
  ChunkWords C;
  read_chunks(C, lb + static_cast<size_t>(b) * kLoadBytes, p);
  // one arrival per warp (the barriers count warps)
  __syncwarp();
  if ((threadIdx.x & 31) == 0) tc::mbar_arrive(tc::smem_u32(&sy->lempty[b]));
  if (issuer && tl.k < src.total) {
    if (!warp_wait(tc::smem_u32(&sy->lempty[b]), lr.round & 1u)) {
      fail_wait(sy, status, 64);
      return false;
    }
    tl.issue(sy, lb, src);
    tl.step(teams, src.n_minor, loads);
  }
  lr.step(teams, loads);
  const int sidx = sr.idx;
  const bool free_stage =
      sr.round == 0 ||
      tc::mbar_wait_ns(tc::smem_u32(&sy->empty[sidx]), (sr.round - 1u) & 1u, kWaitNs);
  if (!__all_sync(0xffffffffu, free_stage)) {
    fail_wait(sy, status, 2);
    return false;
  }
  if constexpr (TMEM) {
    // lanes 32 (warp % 4) ...; chunks 8 h .. 8 h + 7 are columns 32 h .. 32 h + 31 of the stage
    const uint32_t at = a_taddr + (static_cast<uint32_t>((threadIdx.x >> 5) & 3) << 21) +
                        static_cast<uint32_t>(sidx * 64);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      uint32_t r[32];
#pragma unroll
      for (int i = 0; i < 8; ++i)
        chunk_words(C, 8 * h + i, r[4 * i], r[4 * i + 1], r[4 * i + 2], r[4 * i + 3]);
      tc::tmem_st32(at + 32u * h, r);
    }
    tc::tmem_wait_st();
    tc::fence_before_sync();
  } else {
    write_chunks(st + static_cast<size_t>(sidx) * kStageBytes, p, C);
    tc::fence_proxy_async();
  }
  __syncwarp();
  if ((threadIdx.x & 31) == 0) tc::mbar_arrive(tc::smem_u32(&sy->full[sidx]));
  sr.step(teams, stages);
  return true;
}

// A producer warp's whole run: the team's first warp issues the first copies, every warp
// produces the team's stages, and the first warp waits for its last copies before the CTA exits.
template <bool TMEM>
__device__ __forceinline__ void produce_all(Sync* sy, int* status, unsigned char* st,
                                            unsigned char* lb, int loads, int stages,
                                            uint32_t a_taddr, int teams, const StageSource& src) {
  const int warp = threadIdx.x >> 5, team = warp >> 2, p = threadIdx.x & 127;
  const bool issuer = (warp & 3) == 0;
  TeamLoads tl;
  tl.init(team, src.n_minor);
  if (issuer)
    for (int j = 0; j < loads / teams && tl.k < src.total; ++j) {
      tl.issue(sy, lb, src);
      tl.step(teams, src.n_minor, loads);
    }
  Ring lr{team, 0u}, sr{team, 0u};
  for (int64_t k = team; k < src.total && !warp_aborted(sy); k += teams)
    if (!produce<TMEM>(sy, status, st, lb, lr, loads, sr, stages, a_taddr, p, teams, tl, src,
                       issuer))
      break;
  if (issuer) tl.drain(sy, status, teams, loads, team);
}

// Shared set-up of both kernels: zeroed E stages (rows a group leaves unused must hold finite
// values), barriers, tensor memory.
__device__ __forceinline__ void block_setup(Sync* sy, unsigned char* st, int smem_stages,
                                            int stages, int loads, uint32_t tmem_cols,
                                            int mma_warp) {
  const int tid = threadIdx.x;
  for (uint32_t k = tid; k < static_cast<uint32_t>(smem_stages) * kStageBytes / 16u; k += blockDim.x)
    reinterpret_cast<uint4*>(st)[k] = make_uint4(0u, 0u, 0u, 0u);
  if (tid == 0) {
    for (int k = 0; k < stages; ++k) {
      tc::mbar_init(tc::smem_u32(&sy->full[k]), kTeamWarps);
      tc::mbar_init(tc::smem_u32(&sy->empty[k]), 1);
    }
    for (int k = 0; k < loads; ++k) {
      tc::mbar_init(tc::smem_u32(&sy->lfull[k]), 1);
      tc::mbar_init(tc::smem_u32(&sy->lempty[k]), kTeamWarps);
    }
    for (int k = 0; k < 2; ++k) {
      tc::mbar_init(tc::smem_u32(&sy->qfull[k]), 1);
      tc::mbar_init(tc::smem_u32(&sy->qempty[k]), 1);
    }
    tc::mbar_init(tc::smem_u32(&sy->cfull), 1);
    tc::mbar_init(tc::smem_u32(&sy->pass), 1);
    tc::mbar_init(tc::smem_u32(&sy->last), 1);
    sy->abort = 0;
    tc::mbar_init_fence();
  }
  if ((tid >> 5) == mma_warp) tc::tmem_alloc(tc::smem_u32(&sy->tmem), tmem_cols);
  tc::fence_proxy_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
}

// ---- mult: Q[tile] = sum over groups of E[tile][group] C[group] -------------------------------
// A CTA owns `tiles` consecutive tiles, whose accumulators (128 x 32 FP32 each) stay in tensor
// memory, and walks the groups in passes of `gpp` groups whose coefficient rows the loader copies
// into shared memory once the previous pass's MMAs have completed. Output: the Q tiles
// (operand layout of block_multt) and optionally Q in FP64.
// The MMA warp's issue of W consecutive stages: wait for each to be full, then issue their
// K-steps round-robin (neighbouring stages feed different accumulators), then free each stage.
// W is a compile-time constant so that the window's values stay in registers and the MMAs are
// one straight run; the elected lane issues them.
template <int W, bool TMEM_A>
__device__ __forceinline__ bool mult_window(Sync* sy, int* status, Ring& sr, int stages, int& u,
                                            int& gl, int nt, bool later_pass, uint32_t tmem,
                                            uint32_t a_col, unsigned char* st, unsigned char* cf,
                                            uint32_t idesc) {
  int sidx[W];
  uint32_t d[W], a[W];
  uint64_t ad[W], bd[W];
  bool acc[W];
#pragma unroll
  for (int q = 0; q < W; ++q) {
    sidx[q] = sr.idx;
    if (!warp_wait(tc::smem_u32(&sy->full[sidx[q]]), sr.round & 1u)) {
      fail_wait(sy, status, 4);
      return false;
    }
    d[q] = tmem + static_cast<uint32_t>(u * kBlockCols);
    acc[q] = later_pass || gl > 0;
    bd[q] = tc::sdesc(tc::smem_u32(cf + static_cast<size_t>(gl) * kCoefBytes), kCoreK, kCoreMN);
    a[q] = tmem + a_col + static_cast<uint32_t>(sidx[q] * 64);
    ad[q] = tc::sdesc(tc::smem_u32(st + static_cast<size_t>(sidx[q]) * kStageBytes), kCoreK,
                      kCoreMN);
    sr.next(stages);
    if (++u == nt) {
      u = 0;
      ++gl;
    }
  }
  tc::fence_after_sync();
  // K-step j: B moves by 2 core matrices (256 bytes: 16 in the descriptor); A by 256 bytes in
  // shared memory, or by 8 columns in tensor memory
#pragma unroll
  for (int j = 0; j < 8; ++j) {
#pragma unroll
    for (int q = 0; q < W; ++q) {
      if (tc::elect_one()) {
        if constexpr (TMEM_A)
          tc::mma_bf16_ts(d[q], a[q] + 8u * j, bd[q] + 16u * j, idesc, acc[q] || j > 0);
        else
          tc::mma_bf16(d[q], ad[q] + 16u * j, bd[q] + 16u * j, idesc, acc[q] || j > 0);
      }
      __syncwarp();
    }
  }
  if (tc::elect_one()) {
#pragma unroll
    for (int q = 0; q < W; ++q) tc::mma_commit(tc::smem_u32(&sy->empty[sidx[q]]));
  }
  __syncwarp();
  return true;
}

template <int W>
__device__ __forceinline__ bool multt_window(Sync* sy, int* status, Ring& sr, int stages, int& tl,
                                             int& gl, int ng, uint32_t tmem, unsigned char* st,
                                             unsigned char* qb, uint32_t idesc) {
  int sidx[W], qend[W];
  uint32_t d[W];
  uint64_t ad[W], bd[W];
  bool acc[W];
#pragma unroll
  for (int q = 0; q < W; ++q) {
    if (gl == 0 &&
        !warp_wait(tc::smem_u32(&sy->qfull[tl & 1]), static_cast<uint32_t>((tl >> 1) & 1))) {
      fail_wait(sy, status, 16);
      return false;
    }
    sidx[q] = sr.idx;
    if (!warp_wait(tc::smem_u32(&sy->full[sidx[q]]), sr.round & 1u)) {
      fail_wait(sy, status, 4);
      return false;
    }
    d[q] = tmem + static_cast<uint32_t>(gl * kBlockCols);
    acc[q] = tl > 0;
    qend[q] = gl == ng - 1 ? (tl & 1) : -1;
    ad[q] = tc::sdesc(tc::smem_u32(st + static_cast<size_t>(sidx[q]) * kStageBytes), kMnA_LBO,
                      kMnA_SBO);
    bd[q] = tc::sdesc(tc::smem_u32(qb + (tl & 1) * kQBytes), kCoreK, kCoreMN);
    sr.next(stages);
    if (++gl == ng) {
      gl = 0;
      ++tl;
    }
  }
  tc::fence_after_sync();
  // K-step j: A moves by 2 point groups (4096 bytes: 256 in the descriptor), B by 256 bytes
#pragma unroll
  for (int j = 0; j < 8; ++j) {
#pragma unroll
    for (int q = 0; q < W; ++q) {
      if (tc::elect_one())
        tc::mma_bf16(d[q], ad[q] + 256u * j, bd[q] + 16u * j, idesc, acc[q] || j > 0);
      __syncwarp();
    }
  }
  if (tc::elect_one()) {
#pragma unroll
    for (int q = 0; q < W; ++q) {
      tc::mma_commit(tc::smem_u32(&sy->empty[sidx[q]]));
      if (qend[q] >= 0) tc::mma_commit(tc::smem_u32(&sy->qempty[qend[q]]));
    }
  }
  __syncwarp();
  return true;
}

// TMEM_A: the A operand (the stages of E) lives in tensor memory after the accumulators, 64
// columns per stage, instead of in shared memory.
template <bool TMEM_A>
__global__ void __launch_bounds__(kMaxThreads, 1) block_mult_kernel(
    const uint32_t* __restrict__ pc, const BlockHeader* __restrict__ gheader,
    const int2* __restrict__ gslots, const uint16_t* __restrict__ coef, int n_groups, int n_slots, int64_t mpad, int64_t m, int n_tiles,
    int tiles, int gpp, int teams, int stages, int loads, int win, uint32_t tmem_cols, uint16_t* __restrict__ qtiles,
    double* __restrict__ out64, int* __restrict__ status, int f16, const float* __restrict__ scales,
    float pscale, float qfac) {
  extern __shared__ __align__(1024) unsigned char smem[];
  const int smem_stages = TMEM_A ? 0 : stages;
  unsigned char* st = smem;
  unsigned char* lb = st + static_cast<size_t>(smem_stages) * kStageBytes;
  unsigned char* cf = lb + static_cast<size_t>(loads) * kLoadBytes;
  Sync* sy = reinterpret_cast<Sync*>(cf + static_cast<size_t>(gpp) * kCoefBytes);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int t0 = blockIdx.x * tiles;
  const int nt = min(tiles, n_tiles - t0);
  const int passes = static_cast<int>(cdiv(n_groups, gpp));
  const int prod_warps = kTeamWarps * teams, mma_warp = prod_warps, load_warp = prod_warps + 1;
  block_setup(sy, st, smem_stages, stages, loads, tmem_cols, mma_warp);
  const uint32_t tmem = sy->tmem;
  const uint32_t a_col = static_cast<uint32_t>(tiles * kBlockCols);  // first A column (TMEM_A)
  const uint32_t idesc = f16 ? tc::idesc_f16(128, kBlockCols, false, false)
                             : tc::idesc_bf16(128, kBlockCols, false, false);

  if (warp < prod_warps) {
    // the stages of all passes in order (the passes matter only to the MMA and loader warps)
    const StageSource src{pc, gslots, gheader, n_slots, n_groups, nt, 0, t0, true,
                          static_cast<int64_t>(nt) * n_groups};
    produce_all<TMEM_A>(sy, status, st, lb, loads, stages, tmem + a_col, teams, src);
  } else if (warp == mma_warp) {
    Ring sr;
    bool ok = true;
    for (int pass = 0; pass < passes && ok && !warp_aborted(sy); ++pass) {
      const int ng = min(n_groups, pass * gpp + gpp) - pass * gpp;
      if (!warp_wait(tc::smem_u32(&sy->cfull), static_cast<uint32_t>(pass & 1))) {
        fail_wait(sy, status, 1);
        break;
      }
      // stages in the pass: groups outer, tiles inner, so that neighbouring stages feed
      // different accumulators; a window of `win` stages is issued round-robin, one K-step of
      // each in turn (the MMAs of one accumulator are serial, so a lone stage left the tensor
      // cores waiting on each MMA's latency)
      for (int u = 0, gl = 0, left = nt * ng; left > 0 && ok;) {
        if (win >= 3 && left >= 3) {
          ok = mult_window<3, TMEM_A>(sy, status, sr, stages, u, gl, nt, pass > 0, tmem, a_col, st,
                                      cf, idesc);
          left -= 3;
        } else if (win >= 2 && left >= 2) {
          ok = mult_window<2, TMEM_A>(sy, status, sr, stages, u, gl, nt, pass > 0, tmem, a_col, st,
                                      cf, idesc);
          left -= 2;
        } else {
          ok = mult_window<1, TMEM_A>(sy, status, sr, stages, u, gl, nt, pass > 0, tmem, a_col, st,
                                      cf, idesc);
          left -= 1;
        }
      }
      if (tc::elect_one()) tc::mma_commit(tc::smem_u32(&sy->pass));
      __syncwarp();
    }
  } else if (warp == load_warp) {
    // The loader warp copies the coefficient rows of each pass once the MMAs of the pass before
    // have completed (the producers load their own stages).
    auto issue_coef = [&](int pass) {
      const int g0 = pass * gpp, ng = min(n_groups, g0 + gpp) - g0;
      if (tc::elect_one()) {
        const uint32_t cb = tc::smem_u32(&sy->cfull);
        bulk_expect(cb, static_cast<uint32_t>(ng) * kCoefBytes);
        for (int g = 0; g < ng; ++g)
          bulk_copy(tc::smem_u32(cf + static_cast<size_t>(g) * kCoefBytes),
                    coef + static_cast<int64_t>(g0 + g) * 4096, kCoefBytes, cb);
      }
      __syncwarp();
    };
    issue_coef(0);
    int issued = 1;
    for (int pass = 1; pass < passes && !warp_aborted(sy); ++pass) {
      if (!warp_wait(tc::smem_u32(&sy->pass), static_cast<uint32_t>((pass - 1) & 1))) {
        fail_wait(sy, status, 64);
        break;
      }
      issue_coef(pass);
      issued = pass + 1;
    }
    if (!warp_wait(tc::smem_u32(&sy->cfull), static_cast<uint32_t>((issued - 1) & 1)) && lane == 0)
      atomicOr(status, 128);
  }
  // every MMA of the CTA has completed once the last commit has
  if (warp == mma_warp) {
    if (tc::elect_one()) tc::mma_commit(tc::smem_u32(&sy->last));
    __syncwarp();
    if (!warp_wait(tc::smem_u32(&sy->last), 0)) fail_wait(sy, status, 8);
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (!sy->abort && warp < prod_warps) {
    // team t reads tiles t, t + teams, ...; lane = point of the tile
    const int quarter = warp & 3;
    const int p = quarter * 32 + lane;
    for (int u = warp >> 2; u < nt; u += teams) {
      uint32_t r0[16], r1[16];
      const uint32_t ta = tmem + (static_cast<uint32_t>(quarter * 32) << 16) +
                          static_cast<uint32_t>(u * kBlockCols);
      tc::tmem_ld16(ta, r0);
      tc::tmem_ld16(ta + 16, r1);
      tc::tmem_wait_ld();
      const int64_t t = t0 + u;
      const int64_t j = t * 128 + p;
      uint16_t* qt = qtiles ? qtiles + t * 4096 : nullptr;
#pragma unroll
      for (int c = 0; c < kBlockRhs; ++c) {
        const float q = __uint_as_float(r0[c]) + __uint_as_float(r1[c]);
        // FP16: the accumulators hold pscale x scales[c] x Q (powers of two, undone exactly)
        if (out64) {
          const double unscale =
              f16 ? 1.0 / (static_cast<double>(scales[c]) * static_cast<double>(pscale)) : 1.0;
          out64[static_cast<int64_t>(c) * mpad + j] = j < m ? static_cast<double>(q) * unscale : 0.0;
        }
        if (qt) {
          uint16_t hi, lo;
          if (f16)
            split_f16(j < m ? q * qfac : 0.0f, &hi, &lo);
          else
            split_bf16(j < m ? q : 0.0f, &hi, &lo);
          qt[opnd_off(c, p) / 2] = hi;
          qt[opnd_off(c + kBlockRhs, p) / 2] = lo;
        }
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == mma_warp) tc::tmem_dealloc(tmem, tmem_cols);
}

// ---- multT: R[group] = sum over tiles of E[tile][group]^T Q[tile] -----------------------------
// CTA b takes the groups of pass b / streams (up to `gpc` accumulators of 128 rows x 32 FP32 in
// tensor memory) and the tiles of stream b % streams; the loader copies each tile's Q (16-bit,
// operand layout) into one of two buffers ahead of its first stage. The accumulators go out as
// FP64 partial rows of the stream, summed over the streams in order by block_finish_kernel.
// Operand A (E^T, MN-major) core-matrix offsets: along the points (K, leading) and along the
// rows (M, strided).

__global__ void __launch_bounds__(kMaxThreads, 1) block_multt_kernel(
    const uint32_t* __restrict__ pc, const BlockHeader* __restrict__ gheader,
    const int2* __restrict__ gslots, const uint16_t* __restrict__ qtiles, int n_groups, int n_slots, int64_t mpad, int n_tiles, int gpc,
    int streams, int teams, int stages, int loads, int win, uint32_t tmem_cols, int64_t rows,
    double* __restrict__ part, int* __restrict__ status, int f16) {
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* st = smem;
  unsigned char* lb = st + static_cast<size_t>(stages) * kStageBytes;
  unsigned char* qb = lb + static_cast<size_t>(loads) * kLoadBytes;  // two Q tiles
  Sync* sy = reinterpret_cast<Sync*>(qb + 2 * kQBytes);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int pass = blockIdx.x / streams, stream = blockIdx.x % streams;
  const int g0 = pass * gpc, ng = min(gpc, n_groups - g0);
  const int ta = static_cast<int>(static_cast<int64_t>(stream) * n_tiles / streams);
  const int tb = static_cast<int>(static_cast<int64_t>(stream + 1) * n_tiles / streams);
  const int64_t total = ng > 0 ? static_cast<int64_t>(tb - ta) * ng : 0;
  const int prod_warps = kTeamWarps * teams, mma_warp = prod_warps, load_warp = prod_warps + 1;
  block_setup(sy, st, stages, stages, loads, tmem_cols, mma_warp);
  const uint32_t tmem = sy->tmem;
  const uint32_t idesc = f16 ? tc::idesc_f16(128, kBlockCols, true, false)
                             : tc::idesc_bf16(128, kBlockCols, true, false);

  const int nt = tb - ta;
  if (warp < prod_warps && ng > 0) {
    const StageSource src{pc, gslots, gheader, n_slots, n_groups, ng, g0, ta, false, total};
    produce_all<false>(sy, status, st, lb, loads, stages, 0u, teams, src);
  } else if (warp == mma_warp && ng > 0) {
    // windows of `win` consecutive stages (groups inner: different accumulators), issued
    // round-robin one K-step at a time, as in the mult kernel
    Ring sr;
    bool ok = true;
    for (int tl = 0, gl = 0, left = nt * ng; left > 0 && ok && !warp_aborted(sy);) {
      if (win >= 3 && left >= 3) {
        ok = multt_window<3>(sy, status, sr, stages, tl, gl, ng, tmem, st, qb, idesc);
        left -= 3;
      } else if (win >= 2 && left >= 2) {
        ok = multt_window<2>(sy, status, sr, stages, tl, gl, ng, tmem, st, qb, idesc);
        left -= 2;
      } else {
        ok = multt_window<1>(sy, status, sr, stages, tl, gl, ng, tmem, st, qb, idesc);
        left -= 1;
      }
    }
  } else if (warp == load_warp && ng > 0) {
    // Q of tile tl waits only for the MMAs of tile tl - 2 (the producers load their own stages)
    int q_issued = 0;
    for (int tl = 0; tl < nt && !warp_aborted(sy); ++tl) {
      const int b = tl & 1, use = tl >> 1;
      if (use > 0 &&
          !warp_wait(tc::smem_u32(&sy->qempty[b]), static_cast<uint32_t>((use - 1) & 1))) {
        fail_wait(sy, status, 16);
        break;
      }
      if (tc::elect_one()) {
        const uint32_t qbar = tc::smem_u32(&sy->qfull[b]);
        bulk_expect(qbar, kQBytes);
        bulk_copy(tc::smem_u32(qb + b * kQBytes), qtiles + static_cast<int64_t>(ta + tl) * 4096,
                  kQBytes, qbar);
      }
      __syncwarp();
      q_issued = tl + 1;
    }
    for (int tl = q_issued > 2 ? q_issued - 2 : 0; tl < q_issued; ++tl)
      if (!warp_wait(tc::smem_u32(&sy->qfull[tl & 1]), static_cast<uint32_t>((tl >> 1) & 1)) &&
          lane == 0)
        atomicOr(status, 128);
  }
  if (warp == mma_warp) {
    if (tc::elect_one()) tc::mma_commit(tc::smem_u32(&sy->last));
    __syncwarp();
    if (!warp_wait(tc::smem_u32(&sy->last), 0)) fail_wait(sy, status, 8);
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (!sy->abort && warp < prod_warps) {
    const int quarter = warp & 3;
    const int r = quarter * 32 + lane;
    for (int gl = warp >> 2; gl < ng; gl += teams) {
      uint32_t r0[16], r1[16];
      const uint32_t ta2 = tmem + (static_cast<uint32_t>(quarter * 32) << 16) +
                           static_cast<uint32_t>(gl * kBlockCols);
      tc::tmem_ld16(ta2, r0);
      tc::tmem_ld16(ta2 + 16, r1);
      tc::tmem_wait_ld();
      const int64_t row = static_cast<int64_t>(g0 + gl) * 128 + r;
#pragma unroll
      for (int c = 0; c < kBlockRhs; ++c) {
        const double v = total > 0 ? static_cast<double>(__uint_as_float(r0[c])) +
                                         static_cast<double>(__uint_as_float(r1[c]))
                                   : 0.0;
        part[(static_cast<int64_t>(stream) * kBlockRhs + c) * rows + row] = v;
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == mma_warp) tc::tmem_dealloc(tmem, tmem_cols);
}

// out[c][gp] = sum over streams (in order) of the partial rows / (qscale[c] x pscale)
// + scale * add[c][gp] (qscale: the Q tiles' FP16 scales, or null; pscale: the products' scale).
// Threads walk the rows, so that the stream sums read the partial rows coalesced; a row that is
// no grid point's is skipped, and the padding entries gp in [n, npad) are zero.
__global__ void block_finish_kernel(const double* __restrict__ part, int streams, int64_t rows,
                                    const int* __restrict__ row_gp, int64_t n, int64_t npad,
                                    double* __restrict__ out, const double* __restrict__ add,
                                    double scale, const float* __restrict__ qscale,
                                    double pscale) {
  const int64_t total = rows * kBlockRhs;
  for (int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; k < total;
       k += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int c = static_cast<int>(k / rows);
    const int64_t r = k - static_cast<int64_t>(c) * rows;
    const int gp = row_gp[r];
    if (gp < 0) continue;
    double v = 0.0;
    for (int sidx = 0; sidx < streams; ++sidx)
      v += part[(static_cast<int64_t>(sidx) * kBlockRhs + c) * rows + r];
    if (qscale) v /= static_cast<double>(qscale[c]) * pscale;
    const int64_t o = static_cast<int64_t>(c) * npad + gp;
    if (add) v += scale * add[o];
    out[o] = v;
  }
  const int64_t pad = npad - n;
  for (int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
       k < pad * kBlockRhs; k += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int c = static_cast<int>(k / pad);
    out[static_cast<int64_t>(c) * npad + n + (k - static_cast<int64_t>(c) * pad)] = 0.0;
  }
}

// coefficient rows: p column-major FP64 [16][npad] in grid order -> BF16 or FP16 (hi, lo) operand
// blocks (FP16: scaled by scales[c])
template <bool F16>
__global__ void block_coef_kernel(const double* __restrict__ p, int64_t npad,
                                  const int* __restrict__ row_gp, int64_t rows,
                                  uint16_t* __restrict__ coef, const float* __restrict__ scales) {
  const int64_t total = rows * kBlockRhs;
  for (int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; k < total;
       k += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int c = static_cast<int>(k / rows);
    const int64_t r = k - static_cast<int64_t>(c) * rows;
    const int gp = row_gp[r];
    float v = gp >= 0 ? static_cast<float>(p[static_cast<int64_t>(c) * npad + gp]) : 0.0f;
    if constexpr (F16) v *= scales[c];
    uint16_t hi, lo;
    split_pair<F16>(v, &hi, &lo);
    const int64_t g = r >> 7;
    const int rr = static_cast<int>(r & 127);
    coef[g * 4096 + opnd_off(c, rr) / 2] = hi;
    coef[g * 4096 + opnd_off(c + kBlockRhs, rr) / 2] = lo;
  }
}

// Q tiles from a data-side block v column-major FP64 [16][mpad] (zero beyond m; FP16: scaled by
// qscale[c])
template <bool F16>
__global__ void block_qtile_kernel(const double* __restrict__ v, int64_t mpad, int64_t m,
                                   uint16_t* __restrict__ qtiles, const float* __restrict__ qscale) {
  const int64_t total = mpad * kBlockRhs;
  for (int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; k < total;
       k += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int c = static_cast<int>(k / mpad);
    const int64_t j = k - static_cast<int64_t>(c) * mpad;
    float x = j < m ? static_cast<float>(v[k]) : 0.0f;
    if constexpr (F16) x *= qscale[c];
    uint16_t hi, lo;
    split_pair<F16>(x, &hi, &lo);
    const int64_t t = j >> 7;
    const int pp = static_cast<int>(j & 127);
    qtiles[t * 4096 + opnd_off(c, pp) / 2] = hi;
    qtiles[t * 4096 + opnd_off(c + kBlockRhs, pp) / 2] = lo;
  }
}

// packed BF16 or FP16 products of every slot from the materialised float-float products and
// cells; FP16 products are scaled by pscale (a power of two that keeps them out of FP16's
// subnormal range, where they would lose bits)
template <typename CW, bool F16>
__global__ void block_pack_kernel(const float4* __restrict__ pmat, const CW* __restrict__ cmat,
                                  int64_t s_pad, const int* __restrict__ slot_sub, int n_slots,
                                  int64_t m, int64_t mpad, uint32_t* __restrict__ pc, float pscale) {
  constexpr int kBits = sizeof(CW) * 2;
  const int64_t total = static_cast<int64_t>(n_slots) * mpad;
  for (int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; k < total;
       k += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    // k = (tile * n_slots + slot) * 128 + point within the tile
    const int64_t t = k / (static_cast<int64_t>(n_slots) * 128);
    const int64_t rem = k - t * n_slots * 128;
    const int sl = static_cast<int>(rem / 128);
    const int64_t j = t * 128 + (rem & 127);
    uint32_t w = 0u;
    if (j < m) {
      const int64_t at = (j >> 2) * s_pad + slot_sub[sl];
      const float4 q = pmat[at];
      const int lane4 = static_cast<int>(j & 3);
      const float v = lane4 == 0 ? q.x : lane4 == 1 ? q.y : lane4 == 2 ? q.z : q.w;
      const uint32_t cell = (static_cast<uint32_t>(cmat[at]) >> (kBits * lane4)) & ((1u << kBits) - 1u);
      uint16_t bits;
      if constexpr (F16) {
        const __half h = __float2half_rn(v * pscale);
        bits = *reinterpret_cast<const uint16_t*>(&h);
      } else {
        const __nv_bfloat16 b = __float2bfloat16_rn(v);
        bits = *reinterpret_cast<const uint16_t*>(&b);
      }
      w = static_cast<uint32_t>(bits) | (cell << 20);
    }
    pc[k] = w;
  }
}

// *out = max(*out, largest |x| of n floats) as float bits
__global__ void block_absmax_kernel(const float* __restrict__ x, int64_t n,
                                    unsigned* __restrict__ out) {
  unsigned big = 0u;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    big = max(big, __float_as_uint(fabsf(x[i])));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) big = max(big, __shfl_xor_sync(0xffffffffu, big, o));
  if ((threadIdx.x & 31) == 0 && big) atomicMax(out, big);
}

// colmax[c] = max(colmax[c], largest |v[c][i]| for i < count) as float bits (v column-major with
// column stride `pad`); grid (blocks, 16)
__global__ void block_colmax_kernel(const double* __restrict__ v, int64_t pad, int64_t count,
                                    unsigned* __restrict__ colmax) {
  const int c = blockIdx.y;
  const double* col = v + static_cast<int64_t>(c) * pad;
  double big = 0.0;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < count;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    big = fmax(big, fabs(col[i]));
  unsigned b = __float_as_uint(static_cast<float>(big));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) b = max(b, __shfl_xor_sync(0xffffffffu, b, o));
  if ((threadIdx.x & 31) == 0 && b) atomicMax(colmax + c, b);
}

// Power-of-two scales from the column maxima: dst[c] maps column c's largest |value| into
// [2^13, 2^14) (1 for a zero column); with with_q also dst[16 + c] = dst[c] x 2^-shift (the scale
// of the Q tiles block_mult writes). Resets colmax. One warp.
__global__ void block_scale_kernel(unsigned* __restrict__ colmax, float* __restrict__ dst,
                                   int with_q, int shift) {
  const int c = threadIdx.x;
  if (c >= kBlockRhs) return;
  const float big = __uint_as_float(colmax[c]);
  colmax[c] = 0u;
  int e = 0;
  float sc = 1.0f;
  if (big > 0.0f && isfinite(big)) {
    (void)frexpf(big, &e);  // big in [2^(e-1), 2^e)
    sc = ldexpf(1.0f, max(-120, min(120, 14 - e)));
  }
  dst[c] = sc;
  if (with_q) dst[kBlockRhs + c] = ldexpf(sc, -shift);
}

}  // namespace
}  // namespace sgmev

namespace sgmev {
namespace {

// ---- CG on 16 columns -------------------------------------------------------------------------
// Vectors are column-major [16][np]; every dot product reduces in a fixed order (a shared-memory
// tree per block, then the kBlockDotBlocks block sums in block order), so iterations are
// reproducible bit for bit. Scalars (BlockCgScalars offsets) stay on the device.
constexpr int kDotT = 256;

__device__ __forceinline__ double block_tree_sum(double v, double* sh) {
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int w = kDotT / 2; w > 0; w >>= 1) {
    if (static_cast<int>(threadIdx.x) < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  const double r = sh[0];
  __syncthreads();
  return r;
}

__device__ __forceinline__ double sum_parts(const double* __restrict__ part, int k) {
  double s = 0.0;
  for (int b = 0; b < kBlockDotBlocks; ++b) s += part[k * kBlockDotBlocks + b];
  return s;
}

__global__ void __launch_bounds__(kDotT) bcg_dot_kernel(const double* __restrict__ a,
                                                        const double* __restrict__ b, int64_t np,
                                                        double* __restrict__ part) {
  __shared__ double sh[kDotT];
  const int k = blockIdx.y;
  const double* ak = a + static_cast<int64_t>(k) * np;
  const double* bk = b + static_cast<int64_t>(k) * np;
  double v = 0.0;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * kDotT + threadIdx.x; i < np;
       i += static_cast<int64_t>(gridDim.x) * kDotT)
    v += ak[i] * bk[i];
  v = block_tree_sum(v, sh);
  if (threadIdx.x == 0) part[k * kBlockDotBlocks + blockIdx.x] = v;
}

// d = r, e = 0, partial r.r
__global__ void __launch_bounds__(kDotT) bcg_init_kernel(const double* __restrict__ r,
                                                         double* __restrict__ d,
                                                         double* __restrict__ e, int64_t np,
                                                         double* __restrict__ part) {
  __shared__ double sh[kDotT];
  const int k = blockIdx.y;
  const int64_t o = static_cast<int64_t>(k) * np;
  double v = 0.0;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * kDotT + threadIdx.x; i < np;
       i += static_cast<int64_t>(gridDim.x) * kDotT) {
    const double ri = r[o + i];
    d[o + i] = ri;
    e[o + i] = 0.0;
    v += ri * ri;
  }
  v = block_tree_sum(v, sh);
  if (threadIdx.x == 0) part[k * kBlockDotBlocks + blockIdx.x] = v;
}

// delta (slot 0) = delta_0 = the summed partials
__global__ void bcg_set_delta_kernel(const double* __restrict__ part, double* __restrict__ sc) {
  const int k = threadIdx.x;
  if (k < kBlockRhs) {
    const double v = sum_parts(part, k);
    sc[kScDelta + k] = v;
    sc[kScDelta0 + k] = v;
  }
}

// alpha = delta / d.q on active columns; e += alpha d, r -= alpha q; partial r.r
__global__ void __launch_bounds__(kDotT) bcg_update_kernel(
    double* __restrict__ e, double* __restrict__ r, const double* __restrict__ d,
    const double* __restrict__ q, int64_t np, const double* __restrict__ part_dq,
    const double* __restrict__ sc, int cur, double* __restrict__ part_rr) {
  __shared__ double sh[kDotT];
  const int k = blockIdx.y;
  const double delta = sc[kScDelta + cur * kBlockRhs + k];
  const double dq = sum_parts(part_dq, k);
  const bool active = delta > sc[kScTol2 + k] * sc[kScDelta0 + k] && dq != 0.0;
  const double alpha = active ? delta / dq : 0.0;
  const int64_t o = static_cast<int64_t>(k) * np;
  double v = 0.0;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * kDotT + threadIdx.x; i < np;
       i += static_cast<int64_t>(gridDim.x) * kDotT) {
    double ri = r[o + i];
    if (active) {
      e[o + i] = fma(alpha, d[o + i], e[o + i]);
      ri = fma(-alpha, q[o + i], ri);
      r[o + i] = ri;
    }
    v += ri * ri;
  }
  v = block_tree_sum(v, sh);
  if (threadIdx.x == 0) part_rr[k * kBlockDotBlocks + blockIdx.x] = v;
}

// beta = delta_new / delta; d = r + beta d on active columns; delta_new into the other slot
__global__ void __launch_bounds__(kDotT) bcg_direction_kernel(
    const double* __restrict__ r, double* __restrict__ d, int64_t np,
    const double* __restrict__ part_dq, const double* __restrict__ part_rr,
    double* __restrict__ sc, int cur) {
  const int k = blockIdx.y;
  const double delta = sc[kScDelta + cur * kBlockRhs + k];
  const double dq = sum_parts(part_dq, k);
  const bool active = delta > sc[kScTol2 + k] * sc[kScDelta0 + k] && dq != 0.0;
  const double dnew = sum_parts(part_rr, k);
  const double beta = active ? dnew / delta : 0.0;
  const int64_t o = static_cast<int64_t>(k) * np;
  if (active) {
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * kDotT + threadIdx.x; i < np;
         i += static_cast<int64_t>(gridDim.x) * kDotT)
      d[o + i] = fma(beta, d[o + i], r[o + i]);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    // a column whose step was not taken keeps its delta (and stays inactive); d.q = 0 ends it
    sc[kScDelta + (cur ^ 1) * kBlockRhs + k] = active ? dnew : delta;
    sc[kScStalled + k] = (!active && dq == 0.0) ? 1.0 : 0.0;
  }
}

}  // namespace

cudaError_t block_dot(cudaStream_t s, const double* a, const double* b, int64_t np, double* part) {
  bcg_dot_kernel<<<dim3(kBlockDotBlocks, kBlockRhs), kDotT, 0, s>>>(a, b, np, part);
  return cudaGetLastError();
}

cudaError_t block_cg_init(cudaStream_t s, const double* r, double* d, double* e, int64_t np,
                          double* part, double* sc) {
  bcg_init_kernel<<<dim3(kBlockDotBlocks, kBlockRhs), kDotT, 0, s>>>(r, d, e, np, part);
  bcg_set_delta_kernel<<<1, 32, 0, s>>>(part, sc);
  return cudaGetLastError();
}

cudaError_t block_cg_step(cudaStream_t s, double* e, double* r, double* d, const double* q,
                          int64_t np, double* part_dq, double* part_rr, double* sc, int cur) {
  bcg_dot_kernel<<<dim3(kBlockDotBlocks, kBlockRhs), kDotT, 0, s>>>(d, q, np, part_dq);
  bcg_update_kernel<<<dim3(kBlockDotBlocks, kBlockRhs), kDotT, 0, s>>>(e, r, d, q, np, part_dq,
                                                                       sc, cur, part_rr);
  bcg_direction_kernel<<<dim3(kBlockDotBlocks, kBlockRhs), kDotT, 0, s>>>(r, d, np, part_dq,
                                                                          part_rr, sc, cur);
  return cudaGetLastError();
}

}  // namespace sgmev

namespace sgmev {

namespace {
// groups of coefficient rows a mult CTA holds: the shape's count, fewer when the stages leave less
// shared memory (at least one)
// shared-memory stages of E of the mult kernel (none when A lives in tensor memory)
int mult_smem_stages(const BlockShape& sh) { return sh.mult_tmem ? 0 : sh.stages; }
int mult_groups_fit(const BlockShape& sh, int smem_cap) {
  const int64_t room = static_cast<int64_t>(smem_cap) -
                       static_cast<int64_t>(mult_smem_stages(sh)) * kStageBytes -
                       static_cast<int64_t>(sh.loads) * kLoadBytes - static_cast<int64_t>(sizeof(Sync));
  return static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(sh.mult_groups, room / kCoefBytes)));
}
size_t mult_smem(const BlockShape& sh, int groups) {
  return static_cast<size_t>(mult_smem_stages(sh)) * kStageBytes +
         static_cast<size_t>(sh.loads) * kLoadBytes + static_cast<size_t>(groups) * kCoefBytes +
         sizeof(Sync);
}
// tensor-memory columns of the mult kernel: the accumulators, then the A stages
int mult_tmem_need(const BlockShape& sh) {
  return sh.mult_tiles * kBlockCols + (sh.mult_tmem ? sh.stages * 64 : 0);
}
int device_smem_cap() {
  int dev = 0, cap = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&cap, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
    (void)cudaGetLastError();
    return 0;
  }
  return cap;
}
size_t multt_smem(const BlockShape& sh) {
  return static_cast<size_t>(sh.stages) * kStageBytes + static_cast<size_t>(sh.loads) * kLoadBytes +
         2 * kQBytes + sizeof(Sync);
}
uint32_t tmem_cols_for(int accumulators) {
  uint32_t c = 32;
  while (c < static_cast<uint32_t>(accumulators * kBlockCols)) c <<= 1;
  return c;
}
unsigned grid_for(int64_t n, int num_sms) {
  return static_cast<unsigned>(std::max<int64_t>(1, std::min<int64_t>(cdiv(n, 256), 8 * num_sms)));
}
}  // namespace

void block_free(BlockPlan* b) {
  void* ptrs[] = {b->row_gp, b->gp_row, b->gheader, b->gslots, b->pc,     b->coef,
                  b->qtiles, b->part,   b->status,  b->scales, b->colmax};
  for (void* q : ptrs) dev_free(q, b->stream);
  *b = BlockPlan{};
}

bool block_shape_ok(const BlockShape& sh, int smem_cap) {
  return sh.stages >= 2 && sh.stages <= kMaxStages && sh.loads >= 2 && sh.loads <= kMaxLoads &&
         sh.window >= 1 && sh.window <= kMaxWindow && sh.teams >= 1 && sh.teams <= kMaxTeams &&
         sh.teams <= sh.stages && sh.loads % sh.teams == 0 &&
         sh.mult_tiles >= 1 && sh.mult_tiles <= 16 && mult_tmem_need(sh) <= 512 &&
         sh.mult_groups >= 1 && sh.multt_groups >= 1 && sh.multt_groups <= 16 &&
         mult_smem(sh, mult_groups_fit(sh, smem_cap)) <= static_cast<size_t>(smem_cap) &&
         multt_smem(sh) <= static_cast<size_t>(smem_cap);
}

// The multT accumulators (FP32 in tensor memory) take at most about kChainTiles tiles of one
// stream before they are written out as FP64 partial rows: the tensor cores round the running
// sums of a long chain of MMAs toward zero, which biased the sums of 546 tiles by -3e-5 on
// average (and up to -3e-4) in tests against the FP64 products. Streams beyond one CTA per SM
// run as further waves of CTAs; their partial rows take at most kPartBudget bytes.
constexpr int64_t kChainTiles = 64;
constexpr int64_t kPartBudget = int64_t(1) << 30;

static int multt_stream_cap(const BlockPlan& b, int num_sms) {
  const int64_t n_tiles = b.mpad / kBlockTile;
  const int64_t by_budget = std::max<int64_t>(1, kPartBudget / (8 * kBlockRhs * std::max<int64_t>(b.rows, 1)));
  return static_cast<int>(std::max<int64_t>(
      1, std::min<int64_t>(std::min(n_tiles, by_budget),
                           std::max<int64_t>(num_sms, 2 * cdiv(n_tiles, kChainTiles)))));
}

bool block_build(BlockPlan* b, const SubPlan& sub, int64_t m, int64_t mpad, bool f16,
                 cudaStream_t s, int num_sms, std::string* err) {
  block_free(b);
  b->stream = s;
  b->f16 = f16;
  if (!sub.pmat || !sub.cmat || sub.h_sub.empty()) {
    *err = "block products need the materialised subspace products";
    return false;
  }
  if (sub.cmax > kBlockMaxCells) {
    *err = "block products take subspaces of at most 128 cells";
    return false;
  }
  if (mpad % kBlockTile != 0) {
    *err = "block products need the points padded to a multiple of 128";
    return false;
  }
  const int n_sub = sub.n_sub;
  // subspaces by chunk count, largest first; packed into groups of 16 chunks
  std::vector<int> order(n_sub);
  std::iota(order.begin(), order.end(), 0);
  auto chunks = [&](int sidx) { return std::max(1, sub.h_sub[sidx].y / 8); };
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int c) { return chunks(a) > chunks(c); });
  std::vector<int> slot_sub, group_first;
  std::vector<uint16_t> slot_cn;
  int fill = 16;
  for (int sidx : order) {
    const int nch = chunks(sidx);
    if (fill + nch > 16) {
      group_first.push_back(static_cast<int>(slot_sub.size()));
      fill = 0;
    }
    slot_sub.push_back(sidx);
    slot_cn.push_back(static_cast<uint16_t>(fill | (nch << 8)));
    fill += nch;
  }
  const int n_groups = static_cast<int>(group_first.size());
  group_first.push_back(static_cast<int>(slot_sub.size()));
  const int64_t rows = static_cast<int64_t>(n_groups) * kBlockGroupRows;
  // rows <-> grid points
  std::vector<int> pos_gp(static_cast<size_t>(sub.total), -1);
  for (int64_t g = 0; g < sub.n; ++g) pos_gp[sub.h_pos[g]] = static_cast<int>(g);
  std::vector<int> row_gp(static_cast<size_t>(rows), -1), gp_row(static_cast<size_t>(sub.n), 0);
  std::vector<BlockHeader> gheader(static_cast<size_t>(n_groups));
  std::vector<int2> gslots(static_cast<size_t>(n_groups));
  for (int g = 0; g < n_groups; ++g) {
    BlockHeader& hd = gheader[g];
    for (int q = 0; q < 16; ++q) {
      hd.row[q] = 0;  // any row of the group: the shift clears the words
      hd.base[q] = kUnusedBase;
    }
    for (int sl = group_first[g]; sl < group_first[g + 1]; ++sl) {
      const int sidx = slot_sub[sl];
      const int co = slot_cn[sl] & 0xFF, nch = slot_cn[sl] >> 8;
      const int off = sub.h_sub[sidx].x, cells = sub.h_sub[sidx].y;
      for (int c = 0; c < cells; ++c) {
        const int64_t r = static_cast<int64_t>(g) * kBlockGroupRows + (co + c / 8) * 8 + c % 8;
        const int gp = pos_gp[off + c];
        row_gp[r] = gp;
        if (gp >= 0) gp_row[gp] = static_cast<int>(r);
      }
      for (int q = co; q < co + nch; ++q) {
        hd.row[q] = static_cast<int32_t>((sl - group_first[g]) * kSlotRow);
        hd.base[q] = 128 * (q - co);
      }
    }
    gslots[g] = make_int2(group_first[g], group_first[g + 1] - group_first[g]);
  }
  b->n_groups = n_groups;
  b->n_slots = static_cast<int>(slot_sub.size());
  b->rows = rows;
  b->n = sub.n;
  b->m = m;
  b->mpad = mpad;
  b->part_streams = multt_stream_cap(*b, num_sms);
  int* d_slot_sub = nullptr;
  auto alloc = [&](auto** q, size_t bytes) { return dev_malloc(q, bytes, s) == cudaSuccess; };
  auto put = [&](void* dst, const void* src, size_t bytes) {
    return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s) == cudaSuccess;
  };
  bool ok = alloc(&b->row_gp, sizeof(int) * rows) && alloc(&b->gp_row, sizeof(int) * sub.n) &&
            alloc(&b->gheader, sizeof(BlockHeader) * gheader.size()) &&
            alloc(&b->gslots, sizeof(int2) * gslots.size()) &&
            alloc(&d_slot_sub, sizeof(int) * slot_sub.size()) &&
            alloc(&b->pc, sizeof(uint32_t) * static_cast<size_t>(b->n_slots) * mpad) &&
            alloc(&b->coef, kCoefBytes * static_cast<size_t>(n_groups)) &&
            alloc(&b->qtiles, kQBytes * static_cast<size_t>(mpad / kBlockTile)) &&
            alloc(&b->part, sizeof(double) * b->part_streams * kBlockRhs * rows) &&
            alloc(&b->status, sizeof(int)) && alloc(&b->scales, sizeof(float) * 2 * kBlockRhs) &&
            alloc(&b->colmax, sizeof(unsigned) * kBlockRhs);
  ok = ok && put(b->row_gp, row_gp.data(), sizeof(int) * rows) &&
       put(b->gp_row, gp_row.data(), sizeof(int) * sub.n) &&
       put(b->gheader, gheader.data(), sizeof(BlockHeader) * gheader.size()) &&
       put(b->gslots, gslots.data(), sizeof(int2) * gslots.size()) &&
       put(d_slot_sub, slot_sub.data(), sizeof(int) * slot_sub.size()) &&
       cudaMemsetAsync(b->status, 0, sizeof(int), s) == cudaSuccess &&
       cudaMemsetAsync(b->colmax, 0, sizeof(unsigned) * kBlockRhs, s) == cudaSuccess;
  // the largest product: FP16 products are scaled by pe = 2^(14 - e), pmax in [2^(e-1), 2^e), so
  // that the largest lies in [2^13, 2^14) and products down to 2^-27 of it stay normal; the Q tiles
  // take qshift: |Q| <= n_slots x the largest product x the largest coefficient
  unsigned pmax_bits = 0u;
  ok = ok &&
       (block_absmax_kernel<<<grid_for(sub.mat_mpad * sub.s_pad, num_sms), 256, 0, s>>>(
            reinterpret_cast<const float*>(sub.pmat), sub.mat_mpad * sub.s_pad, b->colmax),
        cudaGetLastError() == cudaSuccess) &&
       cudaMemcpyAsync(&pmax_bits, b->colmax, sizeof(unsigned), cudaMemcpyDeviceToHost, s) ==
           cudaSuccess &&
       cudaStreamSynchronize(s) == cudaSuccess &&
       cudaMemsetAsync(b->colmax, 0, sizeof(unsigned) * kBlockRhs, s) == cudaSuccess;
  if (ok) {
    float pmax;
    std::memcpy(&pmax, &pmax_bits, sizeof(pmax));
    int e = 0;
    if (pmax > 0.0f && std::isfinite(pmax)) (void)std::frexp(pmax, &e);
    b->pexp = f16 && pmax > 0.0f ? std::max(-60, std::min(60, 14 - e)) : 0;
    // the accumulators of block_mult reach n_slots x 2^pexp pmax x 2^14; the Q tiles keep 2^14
    const double bound = static_cast<double>(b->n_slots) *
                         std::max(1.0, std::ldexp(static_cast<double>(pmax), b->pexp)) * 16384.0;
    int total = 0;
    while (total < 120 && std::ldexp(16384.0, total) < bound) ++total;
    b->qshift = f16 ? total - b->pexp : 0;
  }
  if (ok) {
    const unsigned blocks = grid_for(static_cast<int64_t>(b->n_slots) * mpad, num_sms);
    const float pscale = std::ldexp(1.0f, b->pexp);
    if (sub.cell_bits == 4) {
      const auto* cm = static_cast<const uint16_t*>(sub.cmat);
      if (f16)
        block_pack_kernel<uint16_t, true><<<blocks, 256, 0, s>>>(sub.pmat, cm, sub.s_pad, d_slot_sub,
                                                                 b->n_slots, m, mpad, b->pc, pscale);
      else
        block_pack_kernel<uint16_t, false><<<blocks, 256, 0, s>>>(sub.pmat, cm, sub.s_pad, d_slot_sub,
                                                                  b->n_slots, m, mpad, b->pc, 1.0f);
    } else {
      const auto* cm = static_cast<const uint32_t*>(sub.cmat);
      if (f16)
        block_pack_kernel<uint32_t, true><<<blocks, 256, 0, s>>>(sub.pmat, cm, sub.s_pad, d_slot_sub,
                                                                 b->n_slots, m, mpad, b->pc, pscale);
      else
        block_pack_kernel<uint32_t, false><<<blocks, 256, 0, s>>>(sub.pmat, cm, sub.s_pad, d_slot_sub,
                                                                  b->n_slots, m, mpad, b->pc, 1.0f);
    }
    ok = cudaGetLastError() == cudaSuccess;
  }
  dev_free(d_slot_sub, s);
  if (!ok) {
    (void)cudaGetLastError();
    block_free(b);
    b->stream = s;
    *err = "block products: allocation or launch failed";
    return false;
  }
  return true;
}

cudaError_t block_mult(BlockPlan& b, cudaStream_t s, const double* p, int64_t npad,
                       double* out64, int num_sms) {
  const BlockShape& sh = b.shape;
  if (b.f16) {
    // per-column scales of the coefficient rows and of the Q tiles this product writes
    block_colmax_kernel<<<dim3(static_cast<unsigned>(std::max<int64_t>(1, std::min<int64_t>(64, cdiv(b.n, 256)))),
                               kBlockRhs),
                          256, 0, s>>>(p, npad, b.n, b.colmax);
    block_scale_kernel<<<1, 32, 0, s>>>(b.colmax, b.scales, 1, b.qshift);
    block_coef_kernel<true><<<grid_for(b.rows * kBlockRhs, num_sms), 256, 0, s>>>(
        p, npad, b.row_gp, b.rows, b.coef, b.scales);
  } else {
    block_coef_kernel<false><<<grid_for(b.rows * kBlockRhs, num_sms), 256, 0, s>>>(
        p, npad, b.row_gp, b.rows, b.coef, nullptr);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const uint32_t cols = tmem_cols_for(cdiv(mult_tmem_need(sh), kBlockCols));
  const int gpp = mult_groups_fit(sh, device_smem_cap());
  // with more than half of the tensor memory per CTA, a second CTA on the SM would only wait for
  // the first one's columns: ask for enough shared memory that it is never placed there
  const size_t smem = cols > 256 ? std::max<size_t>(mult_smem(sh, gpp), 120 * 1024) : mult_smem(sh, gpp);
  auto kern = sh.mult_tmem ? block_mult_kernel<true> : block_mult_kernel<false>;
  e = set_smem_cap(kern, smem);
  if (e != cudaSuccess) return e;
  const int n_tiles = static_cast<int>(b.mpad / kBlockTile);
  const unsigned ctas = static_cast<unsigned>(cdiv(n_tiles, sh.mult_tiles));
  kern<<<ctas, (kTeamWarps * sh.teams + 2) * 32, smem, s>>>(
      b.pc, b.gheader, b.gslots, b.coef, b.n_groups, b.n_slots, b.mpad, b.m, n_tiles, sh.mult_tiles,
      gpp, sh.teams, sh.stages, sh.loads, std::min(sh.window, sh.stages), cols, b.qtiles, out64, b.status,
      b.f16 ? 1 : 0, b.scales, std::ldexp(1.0f, b.pexp), std::ldexp(1.0f, -(b.qshift + b.pexp)));
  return cudaGetLastError();
}

cudaError_t block_multt(BlockPlan& b, cudaStream_t s, const double* v, int64_t npad,
                        double* out64, const double* add, double scale_add, int num_sms) {
  const BlockShape& sh = b.shape;
  cudaError_t e;
  if (v) {
    if (b.f16) {
      block_colmax_kernel<<<dim3(static_cast<unsigned>(std::max<int64_t>(1, std::min<int64_t>(num_sms, cdiv(b.m, 256)))),
                                 kBlockRhs),
                            256, 0, s>>>(v, b.mpad, b.m, b.colmax);
      block_scale_kernel<<<1, 32, 0, s>>>(b.colmax, b.scales + kBlockRhs, 0, 0);
      block_qtile_kernel<true><<<grid_for(b.mpad * kBlockRhs, num_sms), 256, 0, s>>>(
          v, b.mpad, b.m, b.qtiles, b.scales + kBlockRhs);
    } else {
      block_qtile_kernel<false><<<grid_for(b.mpad * kBlockRhs, num_sms), 256, 0, s>>>(
          v, b.mpad, b.m, b.qtiles, nullptr);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  // passes over the groups x streams of tiles: streams of at most about kChainTiles tiles (as
  // many as the partial rows allow), at least one CTA per SM; of those splits the one whose waves
  // of CTAs carry the fewest stages (waves x groups per pass x tiles per stream), at most
  // multt_groups groups per pass and at least kMaxWindow (or all of them): consecutive stages then
  // feed different accumulators, so the MMA window does not change the order of any
  // accumulator's additions.
  const int n_tiles = static_cast<int>(b.mpad / kBlockTile);
  int gpc = sh.multt_groups, streams = 1;
  {
    const int cap = std::max(1, std::min(b.part_streams, std::max(1, n_tiles)));
    int64_t best = -1;
    const int p0 = static_cast<int>(cdiv(b.n_groups, sh.multt_groups));
    for (int p = p0; p <= b.n_groups && p < p0 + 16; ++p) {
      const int g = static_cast<int>(cdiv(b.n_groups, p));
      if (cdiv(b.n_groups, g) != p) continue;  // the same split as fewer passes
      if (g < std::min(kMaxWindow, b.n_groups)) break;
      const int s_lo = static_cast<int>(std::min<int64_t>(
          cap, std::max<int64_t>(std::max(1, num_sms / p), cdiv(n_tiles, kChainTiles))));
      for (int st = s_lo; st <= cap && st < s_lo + 64; ++st) {
        const int64_t waves = cdiv(static_cast<int64_t>(p) * st, num_sms);
        const int64_t cost = waves * g * cdiv(n_tiles, st);
        if (best < 0 || cost < best) {
          best = cost;
          gpc = g;
          streams = st;
        }
      }
    }
  }
  // with more than half of the tensor memory per CTA, a second CTA on the SM would only wait for
  // the first one's columns: ask for enough shared memory that it is never placed there
  const uint32_t cols = tmem_cols_for(gpc);
  const size_t smem = cols > 256 ? std::max<size_t>(multt_smem(sh), 120 * 1024) : multt_smem(sh);
  e = set_smem_cap(block_multt_kernel, smem);
  if (e != cudaSuccess) return e;
  const int passes = static_cast<int>(cdiv(b.n_groups, gpc));
  block_multt_kernel<<<static_cast<unsigned>(passes * streams), (kTeamWarps * sh.teams + 2) * 32,
                       smem, s>>>(
      b.pc, b.gheader, b.gslots, b.qtiles, b.n_groups, b.n_slots, b.mpad, n_tiles, gpc,
      streams, sh.teams, sh.stages, sh.loads, std::min(sh.window, sh.stages), cols, b.rows, b.part, b.status,
      b.f16 ? 1 : 0);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  block_finish_kernel<<<grid_for(b.rows * kBlockRhs, num_sms), 256, 0, s>>>(
      b.part, streams, b.rows, b.row_gp, b.n, npad, out64, add, scale_add,
      b.f16 ? b.scales + kBlockRhs : nullptr, std::ldexp(1.0, b.pexp));
  return cudaGetLastError();
}

cudaError_t block_status(BlockPlan& b, cudaStream_t s, int* host_status) {
  cudaError_t e = cudaMemcpyAsync(host_status, b.status, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e;
}

}  // namespace sgmev
