// Dense fused blocks on the tensor cores (complex64, one HBM pass per block).
//
// The gate fuser (compile.cpp, fusion "dense") multiplies a run of gates on at most
// five qubits into one 2^k x 2^k complex block. Applied with FP32 FMAs, a block of
// k = 4 or 5 qubits costs 8 * 2^k flops per amplitude against 16 bytes of HBM traffic,
// which puts it on the FMA pipe, not HBM. Here the block runs on the 5th-generation
// tensor cores instead (tcgen05.mma, kind::tf32, accumulators in tensor memory):
//
//   * A tile is 4096 amplitudes: every combination of the block's k target bits and
//     the lowest 12 - k other bits. Its HBM footprint is a few contiguous runs of at
//     least 1 KiB (all bits below the highest column bit belong to the tile), moved by
//     the bulk-copy engine (cp.async.bulk, mbarrier completion) into one of six staging
//     buffers in shared memory, and written back from registers by the epilogue warps.
//   * The block is a real GEMM. Column c of the tile (the non-target bits, 128 per
//     MMA) is a row of the A operand holding its 2^k amplitudes as 2^(k+1) reals
//     (re, im interleaved); the B operand is the real form of the block,
//     W[(r,o),(j,i)] = [[Ur, -Ui], [Ui, Ur]], so D[c, 2r+o] is output amplitude (r, c).
//     A lives in tensor memory (row c on lane c, K along the columns), written by the
//     transform warps with tcgen05.st; B is K-major in shared memory with the 128-byte
//     swizzle. Keeping A out of shared memory leaves room for six staging buffers, so
//     several tiles' loads are in flight while earlier tiles are transformed,
//     multiplied and stored.
//   * Precision: every operand is split into a TF32 high part and a TF32 low part
//     (hi = round(x), lo = round(x - hi)); D = Ahi Bhi + Alo Bhi + Ahi Blo accumulates
//     in FP32 in tensor memory, about the accuracy of FP32 arithmetic (3xTF32).
//   * Blocks of fewer than four qubits are widened to four on the host (the identity on
//     the lowest other bits from bit 5 up), so the kernel handles k = 4 and k = 5.
//
// Every wait on an mbarrier is bounded (about a second of wall time); on a timeout the
// kernel records an error code, lets its bulk copies and MMAs drain, frees its tensor
// memory and returns, and the host reports the error.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstring>
#include <vector>

#include "qgpu_internal.h"

namespace qg {
namespace {

constexpr int kTileBits = 12;           // 4096 amplitudes (32 KiB of complex64) per tile
constexpr int kTileAmps = 1 << kTileBits;
constexpr int kThreads = 320;           // transform warps 0-3, epilogue 4-7, loads 8, MMA 9
constexpr int kStageBytes = kTileAmps * 8;
constexpr int kStages = 6;              // staging buffers: tiles whose loads may be in flight
constexpr int kBHalfBytes = 16384;      // one of B hi / B lo at k = 5 (64 x 64 TF32)
// Tensor memory: two buffers of 256 columns, each A hi at [0, 64), A lo at [64, 128)
// and the accumulators D at [128, 192) (both k = 4 with two 128-row blocks of 32
// columns each, and k = 5 with one block of 64 columns).
constexpr int kTmemBufCols = 256;
constexpr int kTmemCols = 2 * kTmemBufCols;
constexpr int kColALo = 64, kColD = 128;

struct DenseTcParams {
  float2* state;
  const float* w;        // B hi then B lo, already in the swizzled K-major layout (2 * bbytes)
  int* err;              // set to a nonzero code when a wait gives up
  int stall;             // failure-path diagnostic: the MMA thread issues nothing
  uint64_t ntiles;
  int k;                 // 4 or 5
  int bbytes;            // bytes of one of B hi / B lo
  // tile-local index bit t (0..11) <-> absolute bit tbit[t]; target or column bit
  int tbit[kTileBits];
  int tgt_of[kTileBits];   // position within j of tile bit t, or -1
  int col_of[kTileBits];   // position within c of tile bit t, or -1
  int runbits;             // the lowest runbits tile bits are bits 0..runbits-1
  // tile index -> base amplitude: runs of the non-tile bits
  int nruns;
  int run_src[64], run_dst[64], run_len[64];
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups 1024 bytes
// apart (stride byte offset), leading byte offset unused (16), descriptor version 1.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)(16u >> 4) << 16;
  d |= (uint64_t)(1024u >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}
// Instruction descriptor of kind::tf32: FP32 accumulator, TF32 A and B, both K-major,
// M = 128, N = n.
__host__ __device__ constexpr uint32_t idesc_tf32(int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}
// D (+)= A B with A read from tensor memory (rows on lanes, K along columns) and B
// from shared memory through its descriptor.
__device__ __forceinline__ void mma_tf32_ts(uint32_t d_tmem, uint32_t a_tmem, uint64_t b, uint32_t idesc,
                                            uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n}\n" ::"r"(d_tmem),
      "r"(a_tmem), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}
// 16 consecutive columns of this thread's lane (tcgen05.st shape 32x32b)
__device__ __forceinline__ void tmem_st16(uint32_t taddr, const float* v) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(
          taddr),
      "f"(v[0]), "f"(v[1]), "f"(v[2]), "f"(v[3]), "f"(v[4]), "f"(v[5]), "f"(v[6]), "f"(v[7]), "f"(v[8]),
      "f"(v[9]), "f"(v[10]), "f"(v[11]), "f"(v[12]), "f"(v[13]), "f"(v[14]), "f"(v[15])
      : "memory");
}
__device__ __forceinline__ float to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// Byte offset of element (row, kk) of a K-major operand with `rows` rows (a multiple
// of 8) in 128-byte swizzled atoms: K-atoms of 32 TF32 values are separate regions of
// rows x 128 bytes; inside one, 8-row groups are 1024 bytes apart and the 16-byte chunk
// index is XORed with the row's position in its group.
__host__ __device__ __forceinline__ uint32_t kmajor_off(int rows, int row, int kk) {
  const int atom = kk >> 5, kin = kk & 31;
  return (uint32_t)(atom * rows * 128 + (row >> 3) * 1024 + (row & 7) * 128 + ((((kin >> 2) ^ (row & 7)) << 4)) +
                    ((kin & 3) << 2));
}

__device__ __forceinline__ uint64_t tile_base(const DenseTcParams& p, uint64_t t) {
  uint64_t b = 0;
  for (int r = 0; r < p.nruns; ++r) b |= ((t >> p.run_src[r]) & ((1ull << p.run_len[r]) - 1)) << p.run_dst[r];
  return b;
}

// The tile's work is a pipeline over four warp roles, each waiting only for its own
// inputs, so the phases of consecutive tiles overlap:
//   load warp (8): refills staging buffer r % 6 with tile r once the transform of tile
//     r - 6 has read it (mbarrier `empty`), by bulk copies completing on `full`;
//   transform warps (0-3): wait for tile r's bytes, split each column's amplitudes into
//     TF32 hi / lo and store them as rows of A in tensor-memory buffer r % 2 (once the
//     MMAs of tile r - 2 have read it, `mma_done`), then release the staging buffer
//     (`empty`) and announce A (`a_full`);
//   MMA warp (9): one thread issues tile r's MMAs into buffer r % 2 once A is there and
//     the epilogue of tile r - 2 has read that buffer's accumulators (`tmem_free`), and
//     commits them to `mma_done`;
//   epilogue warps (4-7): wait for tile r's MMAs, read its accumulators, release the
//     buffer (`tmem_free`) and store the amplitudes straight to HBM (lane c holds
//     column c: consecutive lanes write consecutive amplitudes when the low index bits
//     are column bits).
// Warp w of the transform or epilogue group reaches tensor-memory lanes 32w .. 32w + 31,
// the rows it owns. Every wait is bounded; a warp that gives up raises a shared abort
// flag, which ends every other wait at once, and the load and MMA warps then wait
// (again bounded) for their copies and MMAs in flight before the CTA frees its tensor
// memory. Decisions that lead to a warp-collective instruction are made warp-uniform.
template <int KB>
__global__ void __launch_bounds__(kThreads, 1) k_dense_tc(const __grid_constant__ DenseTcParams p) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  constexpr int D = 1 << KB;               // target combinations
  constexpr int Kp = 2 * D;                // reals per column (K of the GEMM)
  constexpr int Np = Kp;                   // reals per output column (N of the GEMM)
  constexpr int G = (KB == 4) ? 2 : 1;     // 128-column MMA blocks per tile
  constexpr uint32_t idesc = idesc_tf32(Np);
  static_assert(G * Kp == kColALo && 2 * G * Kp == kColD && kColD + G * Np <= kTmemBufCols, "tensor memory map");
  // 1024-aligned regions: B hi, B lo, the staging buffers, then the barriers and tables
  unsigned char* base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  unsigned char* b_hi = base;
  unsigned char* b_lo = b_hi + kBHalfBytes;
  unsigned char* stage = b_lo + kBHalfBytes;
  uint64_t* full = reinterpret_cast<uint64_t*>(stage + kStages * kStageBytes);  // [kStages]
  uint64_t* empty = full + kStages;                                             // [kStages]
  uint64_t* a_full = empty + kStages;                                           // [2]
  uint64_t* mma_done = a_full + 2;                                              // [2]
  uint64_t* tmem_free = mma_done + 2;                                           // [2]
  uint64_t* r_off = tmem_free + 2;                                              // [32]
  uint32_t* jpos = reinterpret_cast<uint32_t*>(r_off + 32);                     // [32]
  uint32_t* tmem_slot = jpos + 32;
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  // the block's real form, hi and lo, already laid out by the host
  for (int i = tid * 4; i < p.bbytes / 4; i += kThreads * 4) {
    *reinterpret_cast<float4*>(b_hi + 4 * i) = *reinterpret_cast<const float4*>(p.w + i);
    *reinterpret_cast<float4*>(b_lo + 4 * i) = *reinterpret_cast<const float4*>(p.w + p.bbytes / 4 + i);
  }
  if (tid < D) {  // target combination j = tid inside a tile: amplitude offset, tile position
    uint64_t o = 0;
    uint32_t pos = 0;
    for (int t = 0; t < kTileBits; ++t)
      if (p.tgt_of[t] >= 0 && ((tid >> p.tgt_of[t]) & 1)) {
        o |= 1ull << p.tbit[t];
        pos |= 1u << t;
      }
    r_off[tid] = o;
    jpos[tid] = pos;
  }
  if (tid == 0) {
    for (int q = 0; q < kStages; ++q) {
      mbar_init(&full[q], 1);
      mbar_init(&empty[q], 4);
    }
    for (int q = 0; q < 2; ++q) {
      mbar_init(&a_full[q], 4);
      mbar_init(&mma_done[q], 1);
      mbar_init(&tmem_free[q], 4);
    }
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_proxy_async();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  const uint64_t t_begin = p.ntiles * blockIdx.x / gridDim.x, t_end = p.ntiles * (blockIdx.x + 1) / gridDim.x;
  const uint64_t count = t_end - t_begin;
  // a bounded wait that also ends when another warp gave up
  auto wait = [&](uint64_t* bar, uint32_t parity) {
    uint64_t t0 = 0;
    for (uint32_t it = 0;; ++it) {
      if (mbar_test(bar, parity)) return true;
      if ((it & 255u) == 0) {
        if (*abort_flag) return false;
        const uint64_t now = global_ns();
        if (t0 == 0) t0 = now;
        else if (now - t0 > 1000000000ull) {
          *abort_flag = 1;
          return false;
        }
      }
    }
  };
  // the same wait, made by every lane, agreed across the warp
  auto wait_warp = [&](uint64_t* bar, uint32_t parity) { return __all_sync(0xffffffffu, wait(bar, parity)) != 0; };
  auto arrive = [&](uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
  };
  const uint32_t lane_base = (uint32_t)(32 * (warp & 3)) << 16;  // this warp's tensor-memory lanes
  uint64_t issued = 0, mmas = 0;  // load warp: tiles whose copies it issued; MMA thread: tiles committed

  if (warp < 4) {
    // ---- transform: tile positions of this thread's columns c = 128 g + 32 warp + lane
    // (the same in every tile; those of the target combinations are the table jpos)
    uint32_t cpos[G];
#pragma unroll
    for (int g = 0; g < G; ++g) {
      const int c = 128 * g + 32 * warp + lane;
      uint32_t pos = 0;
      for (int t = 0; t < kTileBits; ++t)
        if (p.col_of[t] >= 0 && ((c >> p.col_of[t]) & 1)) pos |= 1u << t;
      cpos[g] = pos;
    }
    for (uint64_t r = 0; r < count; ++r) {
      const int s = (int)(r % kStages), b = (int)(r & 1);
      if (!wait_warp(&full[s], (uint32_t)(r / kStages) & 1u)) break;
      if (r >= 2 && !wait_warp(&mma_done[b], (uint32_t)((r - 2) >> 1) & 1u)) break;  // A buffer b is read
      tc_fence_after();
      const float2* st = reinterpret_cast<const float2*>(stage + s * kStageBytes);
      const uint32_t abuf = tmem + lane_base + (uint32_t)(b * kTmemBufCols);
#pragma unroll
      for (int g = 0; g < G; ++g) {
#pragma unroll
        for (int ch = 0; ch < Kp / 16; ++ch) {  // amplitudes j = 8 ch .. 8 ch + 7 of column c
          float hv[16], lv[16];
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const float2 x = st[cpos[g] | jpos[8 * ch + q]];
            const float hr = to_tf32(x.x), hi_ = to_tf32(x.y);
            hv[2 * q] = hr;
            hv[2 * q + 1] = hi_;
            lv[2 * q] = to_tf32(x.x - hr);
            lv[2 * q + 1] = to_tf32(x.y - hi_);
          }
          tmem_st16(abuf + (uint32_t)(g * Kp + 16 * ch), hv);
          tmem_st16(abuf + (uint32_t)(kColALo + g * Kp + 16 * ch), lv);
        }
      }
      __syncwarp();
      if (lane == 0) arrive(&empty[s]);  // this warp's reads of the staging buffer are done
      asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
      tc_fence_before();
      __syncwarp();
      if (lane == 0) arrive(&a_full[b]);
    }
  } else if (warp < 8) {
    // ---- epilogue: lane row = 32 * (warp - 4) + lane of each 128-column block
    const int row = 32 * (warp - 4) + lane;
    uint64_t c_off[2] = {0, 0};
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int c = (G == 2 ? h * 128 : 0) + row;
      for (int t = 0; t < kTileBits; ++t)
        if (p.col_of[t] >= 0 && ((c >> p.col_of[t]) & 1)) c_off[h] |= 1ull << p.tbit[t];
    }
    for (uint64_t r = 0; r < count; ++r) {
      const int b = (int)(r & 1);
      if (!wait_warp(&mma_done[b], (uint32_t)(r >> 1) & 1u)) break;
      tc_fence_after();
      const uint64_t tb = tile_base(p, t_begin + r);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        float v[32];
        // columns kColD + [32h, 32h + 32): block h (k = 4) or outputs 16h..16h+15 (k = 5)
        tmem_ld32(tmem + lane_base + (uint32_t)(b * kTmemBufCols + kColD + 32 * h), v);
        if (h == 1) {  // every accumulator of the buffer is in registers: release it
          tc_fence_before();
          __syncwarp();
          if (lane == 0) arrive(&tmem_free[b]);
        }
        float2* dst = p.state + tb + (G == 2 ? c_off[h] : c_off[0]);
        const int r0 = (G == 2) ? 0 : 16 * h;
#pragma unroll
        for (int q = 0; q < 16; ++q) dst[r_off[r0 + q]] = make_float2(v[2 * q], v[2 * q + 1]);
      }
    }
  } else if (warp == 8) {
    // ---- loads: warp 8's lanes move one run each
    const int nrun = 1 << (kTileBits - p.runbits);  // at most 32: runs are at least 2^7 amplitudes
    const uint32_t run_bytes = (uint32_t)(8u << p.runbits);
    uint64_t run_off = 0;
    if (lane < nrun)
      for (int bb = p.runbits; bb < kTileBits; ++bb)
        if ((lane >> (bb - p.runbits)) & 1) run_off |= 1ull << p.tbit[bb];
    for (; issued < count; ++issued) {
      const int s = (int)(issued % kStages);
      if (issued >= (uint64_t)kStages && !wait_warp(&empty[s], (uint32_t)(issued / kStages - 1) & 1u)) break;
      if (lane == 0) mbar_expect_tx(&full[s], (uint32_t)kStageBytes);
      __syncwarp();
      const uint64_t tb = tile_base(p, t_begin + issued);
      if (lane < nrun)
        bulk_g2s(stage + s * kStageBytes + (size_t)lane * run_bytes, p.state + tb + run_off, run_bytes, &full[s]);
    }
  } else {
    // ---- MMA issue: lane 0 of warp 9 (none under the failure-path diagnostic, so the
    // epilogue's wait for tile 0 runs out)
    if (lane == 0 && !p.stall) {
      const uint64_t dbh = smem_desc(smem_u32(b_hi)), dbl = smem_desc(smem_u32(b_lo));
      for (uint64_t r = 0; r < count; ++r) {
        const int b = (int)(r & 1);
        if (!wait(&a_full[b], (uint32_t)(r >> 1) & 1u)) break;
        if (r >= 2 && !wait(&tmem_free[b], (uint32_t)((r - 2) >> 1) & 1u)) break;  // D of buffer b is read
        tc_fence_after();
        const uint32_t buf = tmem + (uint32_t)(b * kTmemBufCols);
#pragma unroll
        for (int step = 0; step < Kp / 8; ++step) {
          const int atom = step >> 2;
          const uint32_t kin = (uint32_t)(step & 3) * 32u;
          const uint64_t boff = ((uint32_t)(atom * Np * 128) + kin) >> 4;
#pragma unroll
          for (int g = 0; g < G; ++g) {
            const uint32_t d = buf + (uint32_t)(kColD + g * Np);
            const uint32_t ah = buf + (uint32_t)(g * Kp + 8 * step);
            const uint32_t al = buf + (uint32_t)(kColALo + g * Kp + 8 * step);
            mma_tf32_ts(d, ah, dbh + boff, idesc, step > 0 ? 1u : 0u);
            mma_tf32_ts(d, al, dbh + boff, idesc, 1);
            mma_tf32_ts(d, ah, dbl + boff, idesc, 1);
          }
        }
        mma_commit(&mma_done[b]);
        ++mmas;
      }
    }
    __syncwarp();
  }
  __syncthreads();  // every role has left its loop
  if (*abort_flag) {
    // nothing of this CTA may still be in flight when it frees its memory: the last bulk
    // copies issued (they land whether or not a transform consumed them) and the last MMAs
    const uint64_t t0 = global_ns();
    if (warp == 8 && lane == 0)
      for (uint64_t q = issued > (uint64_t)kStages ? issued - kStages : 0; q < issued; ++q)
        while (!mbar_test(&full[q % kStages], (uint32_t)(q / kStages) & 1u) && global_ns() - t0 < 2000000000ull) {
        }
    if (warp == 9 && lane == 0 && mmas)
      while (!mbar_test(&mma_done[(mmas - 1) & 1], (uint32_t)((mmas - 1) >> 1) & 1u) &&
             global_ns() - t0 < 2000000000ull) {
      }
    if (tid == 0) atomicExch(p.err, 1);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
  }
}

size_t dense_tc_smem_bytes() {
  return 1024 + 2 * kBHalfBytes + kStages * kStageBytes + (2 * kStages + 6) * 8 + 32 * 8 + 32 * 4 + 8 + 8;
}

}  // namespace

bool dense_tc_eligible(int n, int dk) { return dk >= 1 && dk <= 5 && n >= kTileBits; }

std::atomic<int> g_dense_tc_stall{0};

// The block's real form for the kernel: a 2^k x 2^k complex block (row-major, (re, im)
// per entry; bit b of a row or column index is absolute bit pos[b]) widened to
// k_eff = max(k, 4) target bits with the identity on other bits (from bit 5 up), then
// W[(r,o),(j,i)] = [[Ur, -Ui], [Ui, Ur]] split into TF32 hi and lo parts and laid out
// K-major with the 128-byte swizzle (N = K = 2^(k_eff+1) rows and columns).
// Returns the widened target bits in tbits_out (ascending) and the floats in w_out.
int dense_tc_prepare(int n, int dk, const int* pos, const double* mat, std::vector<float>* w_out, int* tbits_out) {
  int tb[5], ke = dk;
  for (int i = 0; i < dk; ++i) tb[i] = pos[i];
  // widen with the lowest bits from bit 5 up that are not already targets: the tile's
  // columns then keep index bits 0-4, so the 32 lanes of a warp (32 consecutive columns)
  // read and write 32 consecutive amplitudes (widening with bits 0-2 put each lane's
  // column eight amplitudes from the next: bank conflicts on the staging reads and
  // scattered stores). n >= 12 leaves enough such bits; bits 0-4 are the fallback.
  uint64_t used = 0;
  for (int i = 0; i < dk; ++i) used |= 1ull << pos[i];
  std::vector<int> extra;
  for (int b = 5; b < n && ke + (int)extra.size() < 4; ++b)
    if (!(used & (1ull << b))) extra.push_back(b);
  for (int b = 0; b < 5 && b < n && ke + (int)extra.size() < 4; ++b)
    if (!(used & (1ull << b))) extra.push_back(b);
  for (int b : extra) tb[ke++] = b;
  // sort the widened bits; perm[i] = index in the sorted order of original slot i
  int order[5];
  for (int i = 0; i < ke; ++i) order[i] = i;
  for (int i = 0; i < ke; ++i)
    for (int j = i + 1; j < ke; ++j)
      if (tb[order[j]] < tb[order[i]]) std::swap(order[i], order[j]);
  int sorted_pos_of_slot[5];
  for (int r = 0; r < ke; ++r) sorted_pos_of_slot[order[r]] = r;
  for (int r = 0; r < ke; ++r) tbits_out[r] = tb[order[r]];
  const int De = 1 << ke, D = 1 << dk;
  // widened complex block in sorted-bit indexing
  std::vector<double> U(2 * (size_t)De * De, 0.0);
  auto remap = [&](int idx_slots) {  // index over slots (0..dk-1 original, then extras) -> sorted index
    int out = 0;
    for (int sl = 0; sl < ke; ++sl)
      if ((idx_slots >> sl) & 1) out |= 1 << sorted_pos_of_slot[sl];
    return out;
  };
  for (int ex = 0; ex < (1 << (ke - dk)); ++ex)
    for (int r = 0; r < D; ++r)
      for (int c = 0; c < D; ++c) {
        const int R = remap(r | (ex << dk)), C = remap(c | (ex << dk));
        U[2 * ((size_t)R * De + C)] = mat[2 * ((size_t)r * D + c)];
        U[2 * ((size_t)R * De + C) + 1] = mat[2 * ((size_t)r * D + c) + 1];
      }
  const int K = 2 * De, N = K;
  const int bytes = N * K * 4;
  w_out->assign((size_t)2 * bytes / 4, 0.0f);
  float* whi = w_out->data();
  float* wlo = whi + bytes / 4;
  for (int r = 0; r < De; ++r)
    for (int o = 0; o < 2; ++o)
      for (int j = 0; j < De; ++j)
        for (int i = 0; i < 2; ++i) {
          const double ur = U[2 * ((size_t)r * De + j)], ui = U[2 * ((size_t)r * De + j) + 1];
          const double w = (o == 0) ? (i == 0 ? ur : -ui) : (i == 0 ? ui : ur);
          // TF32: 10 explicit mantissa bits, round to nearest (ties away) on the host
          auto tf32 = [](double x) {
            float f = (float)x;
            uint32_t u;
            std::memcpy(&u, &f, 4);
            if ((u & 0x7f800000u) != 0x7f800000u) u = (u + 0x1000u) & 0xffffe000u;
            std::memcpy(&f, &u, 4);
            return f;
          };
          const float h = tf32(w);
          const float l = tf32(w - (double)h);
          const uint32_t off = kmajor_off(N, 2 * r + o, 2 * j + i) / 4;
          whi[off] = h;
          wlo[off] = l;
        }
  return ke;
}

cudaError_t launch_dense_tc(void* state, int n, int ke, const int* tbits, const float* d_w, int* d_err,
                            cudaStream_t st) {
  if (ke != 4 && ke != 5) return cudaErrorInvalidValue;
  DenseTcParams p;
  std::memset(&p, 0, sizeof(p));
  p.state = (float2*)state;
  p.w = d_w;
  p.err = d_err;
  p.stall = g_dense_tc_stall.load() ? 1 : 0;
  p.k = ke;
  p.bbytes = (2 << ke) * (2 << ke) * 4;
  p.ntiles = 1ull << (n - kTileBits);
  // tile bits: the targets and the lowest 12 - k other bits
  uint64_t tmask = 0;
  for (int i = 0; i < ke; ++i) tmask |= 1ull << tbits[i];
  uint64_t cols = 0;
  int nc = 0;
  for (int b = 0; b < n && nc < kTileBits - ke; ++b)
    if (!(tmask & (1ull << b))) {
      cols |= 1ull << b;
      ++nc;
    }
  const uint64_t all = tmask | cols;
  int t = 0, jn = 0, cn = 0;
  for (int b = 0; b < n; ++b)
    if (all & (1ull << b)) {
      p.tbit[t] = b;
      p.tgt_of[t] = (tmask >> b) & 1 ? jn++ : -1;
      p.col_of[t] = (cols >> b) & 1 ? cn++ : -1;
      ++t;
    }
  int rb = 0;
  while (rb < kTileBits && p.tbit[rb] == rb) ++rb;
  p.runbits = rb;
  if (rb < 1) return cudaErrorInvalidValue;  // the lowest bit always belongs to the tile
  // runs of the remaining bits (tile index bit -> absolute bit)
  int src = 0;
  p.nruns = 0;
  for (int b = 0; b < n;) {
    if (all & (1ull << b)) {
      ++b;
      continue;
    }
    const int dst = b;
    int len = 0;
    while (b < n && !(all & (1ull << b))) {
      ++b;
      ++len;
    }
    p.run_src[p.nruns] = src;
    p.run_dst[p.nruns] = dst;
    p.run_len[p.nruns] = len;
    ++p.nruns;
    src += len;
  }
  static bool attr_set[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  const size_t smem = dense_tc_smem_bytes();
  if (dev >= 0 && dev < 64 && !attr_set[dev]) {
    cudaError_t e = cudaFuncSetAttribute(k_dense_tc<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_dense_tc<5>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    attr_set[dev] = true;
  }
  int sms = kSMCount;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const uint64_t grid = p.ntiles < (uint64_t)sms ? p.ntiles : (uint64_t)sms;
  if (ke == 4) k_dense_tc<4><<<(unsigned)grid, kThreads, smem, st>>>(p);
  else k_dense_tc<5><<<(unsigned)grid, kThreads, smem, st>>>(p);
  count_launch(1);
  return cudaGetLastError();
}

}  // namespace qg
