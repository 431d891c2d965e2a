// gbns_phiw_tc.cu -- the Phi w residual contraction on the 5th-generation tensor cores.
//
// For a tile of 128 points (slice proposals, or dead points for the adjoint) and 128 / 256
// data rows, D[point][row] = w_point . Phi_row is one tcgen05 GEMM with K = P <= 64:
//   * w and Phi are held as TF32 hi + lo parts (x = hi + lo, both rounded to TF32), rows
//     padded with zeros to a multiple of 32 floats, so one K block is one 128-byte row;
//   * one thread issues the TMA loads of the four K-major tiles (128B swizzle, one mbarrier
//     with an expected byte count) and then, per K step of 8, the three products
//     hi*hi + hi*lo + lo*hi as tcgen05.mma kind::tf32 into one FP32 accumulator of
//     128 lanes x 256 columns in tensor memory (3xTF32: fp32-level accuracy);
//   * the four warps read their 32 lanes back with tcgen05.ld (thread = point, 32 rows per
//     load), form r = y - Phi w, and add sum r^2 and sum r y to the point's FP64 totals.
// Every wait is bounded: on time-out the kernel sets GBNS_ERR_WAIT_TIMEOUT, skips the
// epilogue, frees its tensor memory and returns.
#include <cuda.h>
#include <cstdio>
#include <mutex>
#include "gbns_device.cuh"
#include "gbns_launch.h"
#include "gbns_lg.cuh"

namespace gbns {

constexpr int TC_M = 128;                            // points per tile (tensor-memory lanes)
constexpr int TC_N = 256;                            // data rows per tile (tensor-memory columns)
constexpr int TC_KB = 32;                            // floats per 128-byte swizzled row (one K block)
constexpr unsigned TC_A_BYTES = TC_M * TC_KB * 4;    // 16 KB
constexpr unsigned TC_B_BYTES = TC_N * TC_KB * 4;    // 32 KB
constexpr unsigned TC_KB_BYTES = 2 * TC_A_BYTES + 2 * TC_B_BYTES;  // hi + lo of both operands: 96 KB
constexpr long long TC_WAIT_CYCLES = 2000000000ll;   // ~1 s at the maximum SM clock

// Instruction descriptor of tcgen05.mma kind::tf32: D f32 (bits 4-5 = 1), A and B TF32
// (bits 7-9, 10-12 = 2), both K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at
// bits 24-28.
constexpr uint32_t TC_IDESC = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(TC_N >> 3) << 17) |
                              ((uint32_t)(TC_M >> 4) << 24);

struct alignas(128) TcMaps {
  CUtensorMap a_hi, a_lo, b_hi, b_lo;
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor of a K-major tile in the 128-byte swizzle layout written
// by TMA: start address >> 4 (bits 0-13), leading-byte offset 16 B (unused for this layout;
// bits 16-29), stride between 8-row groups 1024 B (bits 32-45), descriptor version 1
// (bit 46), swizzle mode 2 = 128 B (bits 61-63).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(16 >> 4) << 16) | ((uint64_t)(1024 >> 4) << 32) |
         (1ull << 46) | (2ull << 61);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// Waits for phase `parity` of the barrier to complete; false after TC_WAIT_CYCLES.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  const long long t0 = clock64();
  while (true) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
    if (clock64() - t0 > TC_WAIT_CYCLES) return false;
  }
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"((uint64_t)map), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(TC_IDESC), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void tc_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// 32 consecutive fp32 columns of this warp's 32 lanes: thread t gets lane (base lane + t).
__device__ __forceinline__ void tc_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

// One 128-point x 256-row tile.  a_row / b_row: first row of the tile in the point and Phi
// tensor maps; nkb K blocks of 32 are loaded, nk8 K steps of 8 are multiplied; npts points
// and nrows rows are valid.  Must be called by all 128 threads of the CTA.
__device__ void tc_resid_tile(const TcMaps &maps, int a_row, int b_row, int nkb, int nk8, int npts, int nrows,
                              const float *__restrict__ y, double *ss_out, double *ry_out, int *status) {
  extern __shared__ unsigned char tc_dyn[];
  __shared__ __align__(8) unsigned long long bars[2];
  __shared__ uint32_t tmem_slot;
  __shared__ int fail;
  __shared__ float ys[TC_N];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t tiles = (smem_u32(tc_dyn) + 1023u) & ~1023u;  // 1024-byte aligned for the 128B swizzle
  const uint32_t bar_tma = smem_u32(&bars[0]), bar_mma = smem_u32(&bars[1]);

  if (tid == 0) {
    mbar_init(bar_tma, 1);
    mbar_init(bar_mma, 1);
    fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncwarp();
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"((uint32_t)TC_N)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  for (int q = tid; q < TC_N; q += blockDim.x) ys[q] = (q < nrows) ? y[q] : 0.0f;
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;

  if (tid == 0) {
    // lane 0 of warp 0 issues the copies and the MMAs; lanes 1-31 wait for it at __syncwarp
    mbar_expect_tx(bar_tma, (uint32_t)nkb * TC_KB_BYTES);
    for (int kb = 0; kb < nkb; ++kb) {
      const uint32_t base = tiles + (uint32_t)kb * TC_KB_BYTES;
      tma_load_2d(base, &maps.a_hi, kb * TC_KB, a_row, bar_tma);
      tma_load_2d(base + TC_A_BYTES, &maps.a_lo, kb * TC_KB, a_row, bar_tma);
      tma_load_2d(base + 2 * TC_A_BYTES, &maps.b_hi, kb * TC_KB, b_row, bar_tma);
      tma_load_2d(base + 2 * TC_A_BYTES + TC_B_BYTES, &maps.b_lo, kb * TC_KB, b_row, bar_tma);
    }
    if (mbar_wait(bar_tma, 0)) {
      tc_fence_after();
      uint32_t acc = 0;
      for (int k8 = 0; k8 < nk8; ++k8) {
        const int kb = k8 >> 2;
        const uint32_t base = tiles + (uint32_t)kb * TC_KB_BYTES, off = (uint32_t)(k8 & 3) * 32u;
        const uint64_t ah = smem_desc(base + off), al = smem_desc(base + TC_A_BYTES + off);
        const uint64_t bh = smem_desc(base + 2 * TC_A_BYTES + off);
        const uint64_t bl = smem_desc(base + 2 * TC_A_BYTES + TC_B_BYTES + off);
        tc_mma(tmem, al, bh, acc);
        tc_mma(tmem, ah, bl, 1u);
        tc_mma(tmem, ah, bh, 1u);
        acc = 1u;
      }
      tc_commit(bar_mma);
    } else {
      // the copies did not land: report, give them one more bounded wait, release the others
      fail = 1;
      atomicOr(status, (int)GBNS_ERR_WAIT_TIMEOUT);
      mbar_wait(bar_tma, 0);
      mbar_arrive(bar_mma);
    }
  }
  __syncwarp();
  bool ok = mbar_wait(bar_mma, 0);
  ok = __all_sync(0xffffffffu, ok && fail == 0);
  tc_fence_after();
  if (ok) {
    const int pt = warp * 32 + lane;
    const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
    const int nch = (nrows + 31) >> 5;
    double s1 = 0.0, s2 = 0.0;
    for (int ch = 0; ch < nch; ++ch) {
      float v[32];
      tc_ld32(taddr + (uint32_t)(ch * 32), v);
      float p1 = 0.0f, p2 = 0.0f;
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const int row = ch * 32 + j;
        if (row < nrows) {
          const float yy = ys[row];
          const float rr = yy - v[j];
          p1 = fmaf(rr, rr, p1);
          p2 = fmaf(rr, yy, p2);
        }
      }
      s1 += (double)p1;
      s2 += (double)p2;
    }
    if (pt < npts) {
      atomicAdd(&ss_out[pt], s1);
      if (ry_out) atomicAdd(&ry_out[pt], s2);
    }
  } else if (tid == 32) {
    atomicOr(status, (int)GBNS_ERR_WAIT_TIMEOUT);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)TC_N) : "memory");
  }
}

// ------------------------------------------------------------------ sampler step
//
// Persistent, warp-specialised: each CTA walks work units (run, 128-chain tile, range of
// 128-row tiles) with a grid stride.  Warp 0 streams the unit's W tile (hi / lo) and its Phi
// row tiles (hi / lo) through shared memory with TMA, warp 1 issues the 3xTF32 MMAs of each
// row tile into a ring of 128-column accumulators in tensor memory, and warps 2-5 drain the
// accumulators (thread = chain), keep the chain's partial sum of squares in a register over
// the unit's row tiles and add it to the chain's FP64 total once per unit.  Copies, MMAs and
// epilogue of successive row tiles overlap.  Units whose chain tile has no pending proposal
// are skipped by every role alike (the flags are read-only during the launch).
// sum_j (y_j - v_j)^2 over the first n (<= 32) of 32 accumulator columns, in four
// independent FMA chains (j mod 4) so that the reduction does not serialise on FMA latency
__device__ __forceinline__ float sq_resid32(const float *ys, const float *v, int n) {
  float p0 = 0.0f, p1 = 0.0f, p2 = 0.0f, p3 = 0.0f;
  if (n >= 32) {
#pragma unroll
    for (int j = 0; j < 32; j += 4) {
      const float r0 = ys[j] - v[j], r1 = ys[j + 1] - v[j + 1], r2 = ys[j + 2] - v[j + 2], r3 = ys[j + 3] - v[j + 3];
      p0 = fmaf(r0, r0, p0);
      p1 = fmaf(r1, r1, p1);
      p2 = fmaf(r2, r2, p2);
      p3 = fmaf(r3, r3, p3);
    }
  } else {
#pragma unroll
    for (int j = 0; j < 32; j += 4) {
      const float r0 = ys[j] - v[j], r1 = ys[j + 1] - v[j + 1], r2 = ys[j + 2] - v[j + 2], r3 = ys[j + 3] - v[j + 3];
      p0 = j < n ? fmaf(r0, r0, p0) : p0;
      p1 = j + 1 < n ? fmaf(r1, r1, p1) : p1;
      p2 = j + 2 < n ? fmaf(r2, r2, p2) : p2;
      p3 = j + 3 < n ? fmaf(r3, r3, p3) : p3;
    }
  }
  return (p0 + p1) + (p2 + p3);
}

constexpr int SR_ROWS = 128;                       // data rows per tile (accumulator columns)
constexpr unsigned SR_BOX = 128 * TC_KB * 4;       // one K block of 128 rows: 16 KB
constexpr int SR_THREADS = 192;
constexpr uint32_t SR_IDESC = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(SR_ROWS >> 3) << 17) |
                              ((uint32_t)(TC_M >> 4) << 24);

struct alignas(128) SrMaps {
  CUtensorMap w_hi, w_lo, phi_hi, phi_lo;
};

__device__ __forceinline__ void tc_mma_d(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// Bounded wait that also gives up as soon as another role has aborted.
__device__ __forceinline__ bool mbar_wait_or_abort(uint32_t bar, uint32_t parity, const volatile int *abort_flag) {
  const long long t0 = clock64();
  while (true) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
    if (*abort_flag) return false;
    if (clock64() - t0 > TC_WAIT_CYCLES) return false;
  }
}

// Work unit u: false if the run is inactive or the chain tile has no pending proposal (the
// chain step marks such tiles; every warp reaches the same answer).
__device__ __forceinline__ bool sr_unit(const gbns_batch &b, const gbns_lg_bufs &lg, int u, int lane, int &r, int &c0,
                                        int &rt0, int &nrt) {
  const int *it = lg.items_tc + 4 * (size_t)u;
  r = it[0];
  c0 = it[1];
  rt0 = it[2];
  nrt = it[3];
  const gbns_run_state &st = b.state[r];
  if (st.done || st.phase != 1) return false;
  return __shfl_sync(0xffffffffu, lg.tile_pending[lg.tile_base[r] + (c0 >> 7)], 0) != 0;
}

__global__ void __launch_bounds__(SR_THREADS) k_lg_resid_tc(const __grid_constant__ SrMaps maps, gbns_batch b,
                                                            gbns_lg_bufs lg, int nkb_max, int acc_stages) {
  extern __shared__ unsigned char sr_dyn[];
  // 0 w_full, 1 w_empty, 2-3 phi_full, 4-5 phi_empty, 6-9 acc_full, 10-13 acc_empty
  __shared__ __align__(8) unsigned long long bars[14];
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_flag;
  __shared__ float ys[4][SR_ROWS];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t base = (smem_u32(sr_dyn) + 1023u) & ~1023u;
  const int NK = nkb_max;
  auto w_hi = [&](int kb) { return base + (uint32_t)kb * SR_BOX; };
  auto w_lo = [&](int kb) { return base + (uint32_t)(NK + kb) * SR_BOX; };
  auto phi_hi = [&](int p, int kb) { return base + (uint32_t)(2 * NK + p * 2 * NK + kb) * SR_BOX; };
  auto phi_lo = [&](int p, int kb) { return base + (uint32_t)(2 * NK + p * 2 * NK + NK + kb) * SR_BOX; };
  auto bar = [&](int q) { return smem_u32(&bars[q]); };

  pdl_launch_dependents();
  if (tid == 0) {
    mbar_init(bar(0), 1);
    mbar_init(bar(1), 1);
    for (int q = 2; q < 6; ++q) mbar_init(bar(q), 1);
    for (int q = 0; q < 4; ++q) {
      mbar_init(bar(6 + q), 1);
      mbar_init(bar(10 + q), 4);  // one arrival per epilogue warp
    }
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncwarp();
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"((uint32_t)(acc_stages * SR_ROWS))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  const volatile int *ab = &abort_flag;
  const int nunits = lg.num_items_tc;
  pdl_wait_prior_grid();  // the chain step's proposals and tile marks

  if (warp == 0) {
    // ---- producer: W tile per unit, Phi hi / lo per row tile (two stages)
    int wuse = 0, pt = 0;
    for (int u = blockIdx.x; u < nunits; u += gridDim.x) {
      int r, c0, rt0, nrt;
      if (!sr_unit(b, lg, u, lane, r, c0, rt0, nrt)) continue;
      const gbns_run_desc &rd = b.runs[r];
      const int nkb = (rd.D + TC_KB - 1) / TC_KB;
      const int brow = (int)lg.row_base[r];
      int failed = 0;
      if (lane == 0) {
        // Phi row tile t into the next stage (waits until the MMAs have released it)
        auto load_phi = [&](int t) -> bool {
          const int p = pt & 1;
          if (!mbar_wait_or_abort(bar(4 + p), (uint32_t)(((pt >> 1) & 1) ^ 1), ab)) return false;
          mbar_expect_tx(bar(2 + p), 2u * (uint32_t)nkb * SR_BOX);
          const int y0 = brow + (rt0 + t) * SR_ROWS;
          for (int kb = 0; kb < nkb; ++kb) {
            tma_load_2d(phi_hi(p, kb), &maps.phi_hi, kb * TC_KB, y0, bar(2 + p));
            tma_load_2d(phi_lo(p, kb), &maps.phi_lo, kb * TC_KB, y0, bar(2 + p));
          }
          ++pt;
          return true;
        };
        // the first Phi tile goes before the W tile, so it streams while the previous
        // unit's last MMAs (which hold the W buffer) finish
        if (!load_phi(0) || !mbar_wait_or_abort(bar(1), (uint32_t)((wuse & 1) ^ 1), ab)) {
          failed = 1;
        } else {
          mbar_expect_tx(bar(0), 2u * (uint32_t)nkb * SR_BOX);
          const int ar = (int)(rd.shell_off + c0);
          for (int kb = 0; kb < nkb; ++kb) {
            tma_load_2d(w_hi(kb), &maps.w_hi, kb * TC_KB, ar, bar(0));
            tma_load_2d(w_lo(kb), &maps.w_lo, kb * TC_KB, ar, bar(0));
          }
          for (int t = 1; t < nrt; ++t)
            if (!load_phi(t)) {
              failed = 1;
              break;
            }
        }
        if (failed) {
          abort_flag = 1;
          atomicOr(&b.state[r].status, (int)GBNS_ERR_WAIT_TIMEOUT);
        }
      }
      ++wuse;
      if (__shfl_sync(0xffffffffu, failed, 0)) break;
      pt = __shfl_sync(0xffffffffu, pt, 0);
    }
  } else if (warp == 1) {
    // ---- MMA issuer
    int wuse = 0, pt = 0, at = 0;
    for (int u = blockIdx.x; u < nunits; u += gridDim.x) {
      int r, c0, rt0, nrt;
      if (!sr_unit(b, lg, u, lane, r, c0, rt0, nrt)) continue;
      const gbns_run_desc &rd = b.runs[r];
      const int nk8 = (rd.D + 7) / 8;
      int failed = 0;
      if (lane == 0) {
        if (!mbar_wait_or_abort(bar(0), (uint32_t)(wuse & 1), ab)) failed = 1;
        for (int t = 0; t < nrt && !failed; ++t, ++pt, ++at) {
          const int p = pt & 1, a = at % acc_stages;
          if (!mbar_wait_or_abort(bar(2 + p), (uint32_t)((pt >> 1) & 1), ab) ||
              !mbar_wait_or_abort(bar(10 + a), (uint32_t)(((at / acc_stages) & 1) ^ 1), ab)) {
            failed = 1;
            break;
          }
          tc_fence_after();
          const uint32_t d = tmem + (uint32_t)(a * SR_ROWS);
          for (int k8 = 0; k8 < nk8; ++k8) {
            const int kb = k8 >> 2;
            const uint32_t off = (uint32_t)(k8 & 3) * 32u;
            const uint64_t ah = smem_desc(w_hi(kb) + off), al = smem_desc(w_lo(kb) + off);
            const uint64_t bh = smem_desc(phi_hi(p, kb) + off), bl = smem_desc(phi_lo(p, kb) + off);
            tc_mma_d(d, al, bh, SR_IDESC, k8 > 0 ? 1u : 0u);
            tc_mma_d(d, ah, bl, SR_IDESC, 1u);
            tc_mma_d(d, ah, bh, SR_IDESC, 1u);
          }
          tc_commit(bar(6 + a));   // accumulator a full
          tc_commit(bar(4 + p));   // Phi stage p free
          if (t == nrt - 1) tc_commit(bar(1));  // W tile free
        }
        if (failed) {
          abort_flag = 1;
          atomicOr(&b.state[r].status, (int)GBNS_ERR_WAIT_TIMEOUT);
        }
      }
      ++wuse;
      if (__shfl_sync(0xffffffffu, failed, 0)) break;
      pt = __shfl_sync(0xffffffffu, pt, 0);
      at = __shfl_sync(0xffffffffu, at, 0);
    }
  } else {
    // ---- epilogue: warps 2-5 own tensor-memory lane quarters 2, 3, 0, 1
    const int q = warp & 3, ew = warp - 2;
    int at = 0;
    for (int u = blockIdx.x; u < nunits; u += gridDim.x) {
      int r, c0, rt0, nrt;
      if (!sr_unit(b, lg, u, lane, r, c0, rt0, nrt)) continue;
      const gbns_run_desc &rd = b.runs[r];
      const int N = rd.N;
      const float *y = b.fparams + rd.param_off + (size_t)N * rd.D;
      double ssum = 0.0;
      bool ok = true;
      // y of the next row tile is loaded into registers while the current one is processed
      float yn[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int row = rt0 * SR_ROWS + lane + 32 * k;
        yn[k] = row < N ? y[row] : 0.0f;
      }
      for (int t = 0; t < nrt; ++t, ++at) {
        const int a = at % acc_stages;
        const int row0 = (rt0 + t) * SR_ROWS;
        const int nrows = min(SR_ROWS, N - row0);
        __syncwarp();
#pragma unroll
        for (int k = 0; k < 4; ++k) ys[ew][lane + 32 * k] = yn[k];
        __syncwarp();
        if (t + 1 < nrt) {
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const int row = row0 + SR_ROWS + lane + 32 * k;
            yn[k] = row < N ? y[row] : 0.0f;
          }
        }
        ok = mbar_wait_or_abort(bar(6 + a), (uint32_t)((at / acc_stages) & 1), ab);
        ok = __all_sync(0xffffffffu, ok);
        if (!ok) break;
        tc_fence_after();
        const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(a * SR_ROWS);
        const int nch = (nrows + 31) >> 5;
        float part = 0.0f;
        for (int ch = 0; ch < nch; ++ch) {
          float v[32];
          tc_ld32(taddr + (uint32_t)(ch * 32), v);
          part += sq_resid32(&ys[ew][ch * 32], v, nrows - ch * 32);
        }
        ssum += (double)part;
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(bar(10 + a));  // accumulator a drained
      }
      if (!ok) {
        if (lane == 0) {
          abort_flag = 1;
          atomicOr(&b.state[r].status, (int)GBNS_ERR_WAIT_TIMEOUT);
        }
        break;
      }
      const int c = c0 + q * 32 + lane;
      if (c < rd.s) atomicAdd(&lg.ss[rd.shell_off + c], ssum);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"((uint32_t)(acc_stages * SR_ROWS))
                 : "memory");
  }
  // the last CTA to finish clears the pending-tile marks for the next chain step
  __shared__ int last;
  if (tid == 0) {
    __threadfence();
    last = atomicAdd(lg.tc_done, 1) == (int)gridDim.x - 1;
  }
  __syncthreads();
  if (last) {
    for (int q = tid; q < lg.num_tiles; q += blockDim.x) lg.tile_pending[q] = 0;
    if (tid == 0) *lg.tc_done = 0;
  }
}


// ------------------------------------------------------------------ fused shell
//
// One whole lock-step shell of the linear-Gaussian family in one launch.  A thread-block
// cluster of CS CTAs owns one (run, 128-chain tile).  CTA rank q keeps data rows
// [q R, (q + 1) R) of the run's Phi (TF32 hi / lo, K-major 128B-swizzled, loaded once by TMA)
// in shared memory for the whole shell, a 128-chain x R-row accumulator in tensor memory, and
// owns chains q (128 / CS) ... of the tile: one warp per chain, lanes over dimensions, the
// chain logic of k_lg_step with the chain state in registers.  A step:
//   1. every owner warp consumes its chain's residual sum, advances the slice logic and writes
//      the chain's next proposal (one TF32 hi / lo row) into the W tile of every CTA of the
//      cluster (distributed shared memory);
//   2. cluster barrier; the CTAs' counts of active chains travel with it, and the cluster
//      leaves the loop when none is left;
//   3. one thread issues the 3xTF32 tcgen05 MMAs of W (128 chains) x Phi slice (R rows);
//   4. every warp drains a lane quarter x column slice of the accumulator (thread = chain),
//      sums (y - Phi w)^2 over its rows (fp32 over 32-row chunks, the chunks as an fp32
//      pair) and stores the partial sum in the owner CTA's shared memory; cluster barrier.
// The owner adds a chain's partial sums in a fixed butterfly order, so the sum is
// deterministic.  Every
// mbarrier wait is bounded: a CTA whose wait timed out reports it through its active count,
// every CTA of the cluster then leaves at the same barrier, and the run's status gets
// GBNS_ERR_WAIT_TIMEOUT.

struct LfArgs {
  int cs;    // cluster size (CTAs per chain tile)
  int rows;  // data rows per CTA (R)
  int nkb;   // K blocks of 32 floats
  int cpc;   // chains per CTA = warps per CTA (128 / cs)
};

struct alignas(128) LfMaps {
  CUtensorMap phi_hi, phi_lo;
};

__device__ __forceinline__ uint32_t lf_cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

__device__ __forceinline__ void lf_cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// shared::cluster address of the same variable in CTA `rank` of the cluster
__device__ __forceinline__ uint32_t lf_mapa(uint32_t saddr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(saddr), "r"(rank));
  return r;
}

__device__ __forceinline__ void lf_st_v4(uint32_t addr, uint4 v) {
  asm volatile("st.shared::cluster.v4.u32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w)
               : "memory");
}

__device__ __forceinline__ void lf_st_f32x2(uint32_t addr, float a, float b) {
  asm volatile("st.shared::cluster.v2.f32 [%0], {%1, %2};" ::"r"(addr), "f"(a), "f"(b) : "memory");
}

// hi + lo += x (TwoSum of hi and x, the rounding error carried in lo).  GB300 runs FP64 at
// about 1/64 of the FP32 rate, so the step's sums of squares travel as fp32 pairs: each adds
// at most a few units of 2^-48 of relative error, far below the fp32 rounding of the 32-row
// chunk sums they carry.
__device__ __forceinline__ void lf_pair_acc(float &hi, float &lo, float x) {
  float e;
  pair_add(hi, x, hi, e);
  lo += e;
}

__device__ __forceinline__ void lf_st_s32(uint32_t addr, int v) {
  asm volatile("st.shared::cluster.s32 [%0], %1;" ::"r"(addr), "r"(v) : "memory");
}

// byte offset of float k (0..31) of row `row` in a K-major tile with the 128-byte swizzle
// that TMA writes: the 16-byte chunk index is xor-ed with the row's position in its 8-row group
__device__ __forceinline__ uint32_t lf_sw128(int row, int k) {
  return (uint32_t)row * 128u + ((((uint32_t)k >> 2) ^ ((uint32_t)row & 7u)) << 4) + (((uint32_t)k & 3u) << 2);
}

constexpr int LF_ABORT = -(1 << 24);
constexpr int LF_M_TILE = 128;  // chains per cluster tile (tensor-memory lanes)

__global__ void __launch_bounds__(512) k_lg_shell_fused(const __grid_constant__ LfMaps maps, gbns_batch b,
                                                        gbns_lg_bufs lg, LfArgs la) {
  extern __shared__ unsigned char lf_dyn[];
  __shared__ __align__(8) unsigned long long bars[2];  // 0: Phi slice landed, 1: MMAs of a step done
  __shared__ uint32_t tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int CS = la.cs, R = la.rows, NKB = la.nkb, CPC = la.cpc, H = la.cpc / 4;
  const uint32_t rank = lf_cluster_rank();
  const int cl = blockIdx.x / CS;
  const int r = lg.items_fused[2 * cl], tile_c0 = lg.items_fused[2 * cl + 1];
  const gbns_run_desc &rd = b.runs[r];
  gbns_run_state &st = b.state[r];
  if (st.done || st.phase != 1) return;  // the same answer in every CTA of the cluster
  const int P = rd.D, N = rd.N, S = rd.S, K = rd.K, s = rd.s, n = rd.n;
  const int row0 = (int)rank * R;
  const int nrows = max(0, min(R, N - row0));

  // ---- shared memory: Phi slice (hi, lo), W tile (hi, lo), y slice, partial sums, counts
  const uint32_t dyn0 = smem_u32(lf_dyn);
  const uint32_t base = (dyn0 + 1023u) & ~1023u;
  const uint32_t phi_hi = base, phi_lo = base + (uint32_t)(NKB * R * 128);
  const uint32_t w_hi = base + (uint32_t)(2 * NKB * R * 128), w_lo = w_hi + (uint32_t)(NKB * 16384);
  const uint32_t ys_s = w_lo + (uint32_t)(NKB * 16384);
  const uint32_t slots_s = ys_s + (uint32_t)(R * 4);                  // float2 [CS][H][CPC]
  const uint32_t active_s = slots_s + (uint32_t)(CS * H * CPC * 8);   // int [CS]
  // slots: fp32 pairs (hi, lo) [CS][H][CPC]
  auto gptr = [&](uint32_t sa) { return (void *)(lf_dyn + (sa - dyn0)); };
  float *ys = (float *)gptr(ys_s);
  const float2 *slots = (const float2 *)gptr(slots_s);
  const int *active_in = (const int *)gptr(active_s);
  const uint32_t bar_phi = smem_u32(&bars[0]), bar_mma = smem_u32(&bars[1]);

  if (tid == 0) {
    mbar_init(bar_phi, 1);
    mbar_init(bar_mma, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"((uint32_t)R)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  // W tile zeroed (dimensions >= P stay zero); y slice
  for (uint32_t q = (uint32_t)tid; q < (uint32_t)(NKB * 2048); q += blockDim.x)
    *(uint4 *)gptr(w_hi + 16u * q) = make_uint4(0u, 0u, 0u, 0u);
  const float *yrun = b.fparams + rd.param_off + (size_t)N * P;
  for (int q = tid; q < R; q += blockDim.x) ys[q] = q < nrows ? yrun[row0 + q] : 0.0f;
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  const int nbox = (nrows + 127) >> 7;
  if (tid == 0 && nbox > 0) {
    mbar_expect_tx(bar_phi, (uint32_t)(2 * NKB * nbox) * SR_BOX);
    const int brow = (int)lg.row_base[r] + row0;
    for (int kb = 0; kb < NKB; ++kb)
      for (int i = 0; i < nbox; ++i) {
        const uint32_t o = (uint32_t)(kb * R * 128 + i * 16384);
        tma_load_2d(phi_hi + o, &maps.phi_hi, kb * TC_KB, brow + 128 * i, bar_phi);
        tma_load_2d(phi_lo + o, &maps.phi_lo, kb * TC_KB, brow + 128 * i, bar_phi);
      }
  }
  int abort_local = 0;
  if (nbox > 0) abort_local = __syncthreads_or(!mbar_wait(bar_phi, 0)) ? 1 : 0;

  // ---- the owned chain (warp): seed point, keys (k_lg_init)
  const float *liveL = b.live_L[st.parity] + rd.live_off;
  const float Lstar = liveL[rd.s - 1];
  const int crow = (int)rank * CPC + warp;  // chain row in the tile
  const int c = tile_c0 + crow;
  const int pa_ = lane, pb_ = lane + 32;
  const bool ha = pa_ < P, hb = pb_ < P;
  int flags = LG_DONE;
  float ua = 0.f, la_ = 0.f, ub = 0.f, lb = 0.f, da = 0.f, db = 0.f;
  int j = 0, total = 0, in_slice = 0;
  float left = 0.f, right = 0.f, t = 0.f, alpha = 0.5f, logL0 = 0.f;
  Key ck = {0u, 0u}, after_key = {0u, 0u}, dir_key = {0u, 0u}, slices_key = {0u, 0u};
  if (c < s) {
    int lo = 0, hi = n;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (liveL[mid] > Lstar) hi = mid; else lo = mid + 1;
    }
    const int m = n - lo;
    const Key k0 = {st.key[0], st.key[1]};
    const Key sample_key = fold(fold(k0, 0u), 1u);
    const Key kc = fold(sample_key, (uint32_t)c);
    const Key chain_key = fold(kc, 0u), seed_key = fold(kc, 1u);
    int idx = 0;
    if (m > 0) {
      const uint64_t M52 = bits64(seed_key, 0u) >> 12;
      const uint64_t q = (1ull << 52) - M52;
      const uint64_t lo64 = (uint64_t)m * q, hi64 = __umul64hi((uint64_t)m, q);
      uint64_t kk = (hi64 << 12) | (lo64 >> 52);
      if (lo64 & ((1ull << 52) - 1)) kk += 1;
      idx = (n - m) + (int)kk - 1;
    }
    const double *liveU = (const double *)(b.live_U[st.parity] + rd.liveU_off);
    if (ha) pair_from_double(liveU[(size_t)idx * P + pa_], ua, la_);
    if (hb) pair_from_double(liveU[(size_t)idx * P + pb_], ub, lb);
    logL0 = liveL[idx];
    dir_key = fold(chain_key, 0u);
    slices_key = fold(chain_key, 1u);
    flags = LG_START | LG_NEED_DIR;
  }
  const float *fp = b.fparams + rd.param_off;
  const float sigma = fp[(size_t)N * P + N];
  const float inv2s2 = 0.5f / (sigma * sigma);
  const int *kind = b.prior_kind + rd.prior_off;
  const float *pra = b.prior_a + rd.prior_off, *prb = b.prior_b + rd.prior_off;
  lf_cluster_sync();  // every CTA initialised before the first remote store

  // ---- speculation.  Both possible continuations of a chain's next step are fixed by its
  // keys, so each warp computes them while the cluster exchanges partial sums, off the critical
  // path: the direction of the next slice (the normals of the current slice's after_key, lanes
  // over dimensions), the keys and uniform of the next slice's first pick (B' = split(slices_key)[j],
  // then run / t / after keys), and the keys and uniform of the next shrink step (from the
  // current carry key).  The chain step then only selects.
  // The next slice's continuation (its direction normals from this slice's after_key, its base
  // key B' and the keys and uniform of its first pick) is the same for every step of a slice:
  // it is derived at the slice's first step (spec_j records for which slice) and reused; only
  // the shrink continuation changes from step to step.
  float sa_va = 0.f, sa_vb = 0.f, sa_nrm = 1.f, sa_u = 0.f, sr_u = 0.f;
  Key sa_ck = {0u, 0u}, sa_after = {0u, 0u}, sr_ck = {0u, 0u};
  int spec_j = -1;
  auto speculate = [&](Key next_dir_key, int next_j, Key cur_ck) {
    uint32_t x0, x1;
    if (next_j != spec_j) {
      spec_j = next_j;
      if (P > 1) {
        sa_va = ha ? normal_from_bits(bits64(next_dir_key, (uint32_t)pa_)) : 0.0f;
        sa_vb = hb ? normal_from_bits(bits64(next_dir_key, (uint32_t)pb_)) : 0.0f;
        sa_nrm = sqrtf(warp_sum(fmaf(sa_va, sa_va, sa_vb * sa_vb)));
      }
      // B' = fold(slices_key, next_j); then lanes 0-2: its run, t and after keys (counters
      // 0, 2, 3); then the first pick's 64 random bits
      threefry2x32(slices_key.k0, slices_key.k1, 0u, (uint32_t)next_j, x0, x1);
      const uint32_t c2 = lane == 1 ? 2u : (lane == 2 ? 3u : 0u);
      threefry2x32(x0, x1, 0u, c2, x0, x1);
      sa_ck.k0 = __shfl_sync(0xffffffffu, x0, 0);
      sa_ck.k1 = __shfl_sync(0xffffffffu, x1, 0);
      const Key tka = {__shfl_sync(0xffffffffu, x0, 1), __shfl_sync(0xffffffffu, x1, 1)};
      sa_after.k0 = __shfl_sync(0xffffffffu, x0, 2);
      sa_after.k1 = __shfl_sync(0xffffffffu, x1, 2);
      threefry2x32(tka.k0, tka.k1, 0u, 0u, x0, x1);
      sa_u = uniform01(((uint64_t)x0 << 32) | (uint64_t)x1);
    }
    // the shrink continuation -- lane 1: carry fold(ck, 0); lane 2: t key fold(ck, 1); then
    // the t key's 64 random bits
    threefry2x32(cur_ck.k0, cur_ck.k1, 0u, lane == 2 ? 1u : 0u, x0, x1);
    sr_ck.k0 = __shfl_sync(0xffffffffu, x0, 1);
    sr_ck.k1 = __shfl_sync(0xffffffffu, x1, 1);
    const Key tkr = {__shfl_sync(0xffffffffu, x0, 2), __shfl_sync(0xffffffffu, x1, 2)};
    threefry2x32(tkr.k0, tkr.k1, 0u, 0u, x0, x1);
    sr_u = uniform01(((uint64_t)x0 << 32) | (uint64_t)x1);
  };
  if (!(flags & LG_DONE)) speculate(dir_key, 0, ck);

  const int NMMA = R < 256 ? R : 256;
  const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(NMMA >> 3) << 17) | ((uint32_t)(TC_M >> 4) << 24);
  const int nk8 = (P + 7) >> 3;
  const int qd = warp & 3, hs = warp >> 2;  // accumulator lane quarter and column slice of this warp
  uint32_t mma_phase = 0;
  bool mma_pending = false;
  for (long long step = 0;; ++step) {
    // ---- 1. chain step of the owned chain (k_lg_step's logic, continuations precomputed)
    bool wrote = false;
    if (!(flags & LG_DONE)) {
      bool start_now = true;  // the first pick of slice 0
      if (flags & LG_PENDING) {
        // this chain's residual sum: its partial sums from every CTA and column slice (one per
        // lane), added in a fixed butterfly order
        const float2 part_in = lane < CS * H ? slots[lane * CPC + warp] : make_float2(0.0f, 0.0f);
        float shi = part_in.x, slo = part_in.y;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          const float ohi = __shfl_xor_sync(0xffffffffu, shi, o), olo = __shfl_xor_sync(0xffffffffu, slo, o);
          float e;
          pair_add(shi, ohi, shi, e);
          slo = (slo + olo) + e;
        }
        // -(shi + slo) * inv2s2, the product's rounding error carried by an FMA
        const float prod = shi * inv2s2;
        float logL = -(prod + fmaf(slo, inv2s2, fmaf(shi, inv2s2, -prod)));  // relative to log_L_offset
        if (logL != logL) logL = -INFINITY;
        ++total;
        ++in_slice;
        const bool accept = (logL > Lstar) || ((logL0 == Lstar) && (logL == Lstar));
        start_now = false;
        if (accept || in_slice >= b.max_evals_per_slice) {
          if (!accept) flags |= LG_FAILED;
          pair_add(ua, fmaf(t, da, la_), ua, la_);
          pair_add(ub, fmaf(t, db, lb), ub, lb);
          logL0 = logL;
          const int ph = j - (S - 1 - K);
          if (K > 0 && ph >= 0 && j < S - 1) {
            double *phU = (double *)(b.ph_U + rd.phU_off) + ((size_t)c * K + ph) * P;
            if (ha) phU[pa_] = (double)ua + (double)la_;
            if (hb) phU[pb_] = (double)ub + (double)lb;
            if (lane == 0) b.ph_L[rd.phL_off + (size_t)c * K + ph] = logL;
          }
          ++j;
          if (j < S) start_now = true;
          else flags |= LG_DONE;
        }
        flags &= ~LG_PENDING;
      }
      if (flags & LG_DONE) {
        double *nu = (double *)(b.new_U + rd.newU_off) + (size_t)c * P;
        if (ha) nu[pa_] = (double)ua + (double)la_;
        if (hb) nu[pb_] = (double)ub + (double)lb;
        if (lane == 0) {
          b.new_L[rd.shell_off + c] = logL0;
          b.new_E[rd.shell_off + c] = total;
          if (flags & LG_FAILED) atomicOr(&st.status, (int)GBNS_ERR_SHRINK_BUDGET);
        }
      } else {
        float u;
        if (start_now) {
          if (P == 1) {
            da = 1.0f;
          } else {
            da = sa_va / sa_nrm;
            db = sa_vb / sa_nrm;
          }
          ck = sa_ck;
          after_key = sa_after;
          u = sa_u;
          alpha = lg_alpha(j, S);
          float t1r = INFINITY, t1l = -INFINITY, t0r = INFINITY, t0l = -INFINITY;
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const bool have = h ? hb : ha;
            if (have) {
              const float uu = h ? ub : ua, ll = h ? lb : la_, dd = h ? db : da;
              const float t1 = ((1.0f - uu) - ll) / dd, t0 = -(uu + ll) / dd;
              t1r = fminf(t1r, t1 >= 0.f ? t1 : INFINITY);
              t1l = fmaxf(t1l, t1 <= 0.f ? t1 : -INFINITY);
              t0r = fminf(t0r, t0 >= 0.f ? t0 : INFINITY);
              t0l = fmaxf(t0l, t0 <= 0.f ? t0 : -INFINITY);
            }
          }
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) {
            t1r = fminf(t1r, __shfl_xor_sync(0xffffffffu, t1r, o));
            t1l = fmaxf(t1l, __shfl_xor_sync(0xffffffffu, t1l, o));
            t0r = fminf(t0r, __shfl_xor_sync(0xffffffffu, t0r, o));
            t0l = fmaxf(t0l, __shfl_xor_sync(0xffffffffu, t0l, o));
          }
          right = fminf(t0r, t1r);
          left = fmaxf(t0l, t1l);
          in_slice = 0;
        } else {
          ck = sr_ck;
          u = sr_u;
          if (t < 0.f) left = t;
          if (t > 0.f) right = t;
          if (rd.midpoint) {
            if (t < 0.f) left = alpha * left;
            if (t > 0.f) right = alpha * right;
          }
        }
        t = fmaf(u, right - left, left);
        // the proposal w as a TF32 hi / lo row of the W tile
        if (ha) {
          const float w = prior_quantile_pair(kind[pa_], pra[pa_], prb[pa_], ua, fmaf(t, da, la_));
          float h, l;
          tf32_split(w, h, l);
          *(float *)gptr(w_hi + lf_sw128(crow, pa_)) = h;
          *(float *)gptr(w_lo + lf_sw128(crow, pa_)) = l;
        }
        if (hb) {
          const float w = prior_quantile_pair(kind[pb_], pra[pb_], prb[pb_], ub, fmaf(t, db, lb));
          float h, l;
          tf32_split(w, h, l);
          *(float *)gptr(w_hi + 16384u + lf_sw128(crow, lane)) = h;
          *(float *)gptr(w_lo + 16384u + lf_sw128(crow, lane)) = l;
        }
        flags |= LG_PENDING;
        wrote = true;
      }
    }
    __syncwarp();
    if (wrote) {
      if (lane < 16 * NKB) {
        // copy the row (hi and lo, NKB blocks of 128 bytes) to the other CTAs of the cluster
        const int blk = lane >> 3, chunk = lane & 7;
        const uint32_t off = ((blk & 1) ? w_lo : w_hi) + (uint32_t)(blk >> 1) * 16384u + (uint32_t)crow * 128u +
                             (uint32_t)chunk * 16u;
        const uint4 v = *(const uint4 *)gptr(off);
        for (int q = 0; q < CS; ++q)
          if (q != (int)rank) lf_st_v4(lf_mapa(off, (uint32_t)q), v);
      }
      // the tensor cores of every CTA read the row through the async proxy
      asm volatile("fence.proxy.async.shared::cluster;" ::: "memory");
    }
    const int act = __syncthreads_count(lane == 0 && !(flags & LG_DONE));
    if (tid < CS) lf_st_s32(lf_mapa(active_s + 4u * rank, (uint32_t)tid), abort_local ? LF_ABORT : act);
    lf_cluster_sync();  // (A) W tiles and active counts complete in every CTA
    int total_active = 0;
    for (int q = 0; q < CS; ++q) total_active += active_in[q];
    if (total_active <= 0 || step >= lg.max_steps) {
      if (tid == 0 && rank == 0) {
        if (total_active < 0) atomicOr(&st.status, (int)GBNS_ERR_WAIT_TIMEOUT);
        else if (total_active > 0) atomicOr(&st.status, (int)GBNS_ERR_SHRINK_BUDGET);
      }
      break;
    }
    // ---- 2. 3xTF32 MMAs: accumulator[chain][row] = W[chain] . Phi[row] over this CTA's rows
    if (nbox > 0 && tid == 0) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      tc_fence_after();
      for (int nc = 0; nc * NMMA < nbox * 128; ++nc) {
        const uint32_t d = tmem + (uint32_t)(nc * NMMA);
        for (int k8 = 0; k8 < nk8; ++k8) {
          const int kb = k8 >> 2;
          const uint32_t koff = (uint32_t)(k8 & 3) * 32u;
          const uint32_t wo = (uint32_t)kb * 16384u + koff;
          const uint32_t po = (uint32_t)(kb * R * 128 + nc * NMMA * 128) + koff;
          const uint64_t ah = smem_desc(w_hi + wo), al = smem_desc(w_lo + wo);
          const uint64_t bh = smem_desc(phi_hi + po), bl = smem_desc(phi_lo + po);
          tc_mma_d(d, al, bh, idesc, k8 > 0 ? 1u : 0u);
          tc_mma_d(d, ah, bl, idesc, 1u);
          tc_mma_d(d, ah, bh, idesc, 1u);
        }
      }
      tc_commit(bar_mma);
    }
    // ---- 3. epilogue: this warp's 32 chains x its column slice
    float part = 0.0f, part_lo = 0.0f;
    if (nbox > 0) {
      bool ok = mbar_wait(bar_mma, mma_phase);
      ok = __syncthreads_and(ok);
      if (!ok) {
        abort_local = 1;
        mma_pending = true;  // the phase stays the one still owed
      } else {
        mma_phase ^= 1u;
        tc_fence_after();
        const int cw = R / H;
        const int cbeg = hs * cw, cend = min(cbeg + cw, nrows);
        const uint32_t taddr = tmem + ((uint32_t)(qd * 32) << 16);
        for (int col = cbeg; col < cend; col += 32) {
          float v[32];
          tc_ld32(taddr + (uint32_t)col, v);
          lf_pair_acc(part, part_lo, sq_resid32(ys + col, v, cend - col));
        }
      }
    }
    {
      const int row_c = qd * 32 + lane;  // chain row of this thread's accumulator lane
      const int owner = row_c / CPC, lc = row_c - owner * CPC;
      lf_st_f32x2(lf_mapa(slots_s + 8u * (uint32_t)(((int)rank * H + hs) * CPC + lc), (uint32_t)owner), part,
                  part_lo);
    }
    tc_fence_before();
    // (B) partial sums complete in their owners; the continuations of the next step are
    // computed between the arrival and the wait
    asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
    if (flags & LG_PENDING) speculate(after_key, j + 1, ck);
    asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
  }
  // a timed-out MMA may still be in flight: give it one more bounded wait before the
  // tensor memory is released
  if (mma_pending && tid == 0) mbar_wait(bar_mma, mma_phase);
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)R) : "memory");
  }
  lf_cluster_sync();
}

// Adjoint: all dead points (blockIdx.x: 128-point tile) against all rows (blockIdx.y).
__global__ void __launch_bounds__(128) k_adj_resid_tc(const __grid_constant__ TcMaps maps, long long M, int P, int N,
                                                      const float *y, double *ss, double *ry, int *status) {
  const long long p0 = (long long)blockIdx.x * TC_M;
  const int row0 = blockIdx.y * TC_N;
  tc_resid_tile(maps, (int)p0, row0, (P + TC_KB - 1) / TC_KB, (P + 7) / 8, (int)min((long long)TC_M, M - p0),
                min(TC_N, N - row0), y + row0, ss + p0, ry + p0, status);
}

// Phi of every run -> TF32 hi / lo rows of 64 floats (zero beyond P).
__global__ void k_split_phi(gbns_batch b, gbns_lg_bufs lg) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= lg.total_rows * 64) return;
  const long long grow = q >> 6;
  const int k = (int)(q & 63);
  int lo = 0, hi = b.num_runs;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (lg.row_base[mid] <= grow) lo = mid; else hi = mid;
  }
  const gbns_run_desc &rd = b.runs[lo];
  const long long row = grow - lg.row_base[lo];
  float h = 0.0f, l = 0.0f;
  if (row < rd.N && k < rd.D) tf32_split(b.fparams[rd.param_off + row * rd.D + k], h, l);
  lg.Phi_hi[q] = h;
  lg.Phi_lo[q] = l;
}

// Dead points for the adjoint: w = tau * sqrt(2) * erfinv(2u - 1) (the Normal(0, tau^2)
// quantile), and Phi, both as TF32 hi/lo rows of ld floats.
__global__ void k_adj_split(const double *U, long long M, int P, const float *Phi, int N, float tau, int ld,
                            float *w_hi, float *w_lo, float *phi_hi, float *phi_lo) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long nw = M * ld, np = (long long)N * ld;
  if (q >= nw + np) return;
  float h = 0.0f, l = 0.0f;
  if (q < nw) {
    const long long i = q / ld;
    const int k = (int)(q % ld);
    if (k < P) tf32_split(tau * ndtri_from_double(U[i * P + k]), h, l);
    w_hi[q] = h;
    w_lo[q] = l;
  } else {
    const long long e = q - nw, row = e / ld;
    const int k = (int)(e % ld);
    if (k < P) tf32_split(Phi[row * P + k], h, l);
    phi_hi[e] = h;
    phi_lo[e] = l;
  }
}

// ----------------------------------------------------------------------------- host side

namespace {

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
  });
  return fn;
}

// rows x ld fp32 matrix (row stride ld * 4 bytes), boxes of 32 floats x box_rows rows,
// 128-byte swizzle, zero fill outside.
bool encode_rows(CUtensorMap *m, const float *base, long long rows, int ld, int box_rows) {
  EncodeTiledFn fn = encode_fn();
  if (!fn || !base || rows < 1 || (ld != 32 && ld != 64) || ((uintptr_t)base & 15)) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)ld, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)ld * 4};
  const cuuint32_t box[2] = {(cuuint32_t)TC_KB, (cuuint32_t)box_rows};
  const cuuint32_t es[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void *)base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The dynamic shared-memory limit of the two tile kernels, raised once per device.
cudaError_t set_smem_attrs() {
  static std::mutex mu;
  static bool done[64] = {false};
  int dev = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err != cudaSuccess) return err;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(mu);
  if (done[dev]) return cudaSuccess;
  const int bytes = 2 * (int)TC_KB_BYTES + 1024;  // two K blocks: 6 x 2 x 16 KB (sampler) or 2 x 96 KB (adjoint)
  err = cudaFuncSetAttribute(k_lg_resid_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (err == cudaSuccess) err = cudaFuncSetAttribute(k_adj_resid_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (err == cudaSuccess) done[dev] = true;
  return err;
}

}  // namespace

cudaError_t lg_tc_prepare(const gbns_batch &b, const gbns_lg_bufs &lg, cudaStream_t s) {
  cudaError_t e = set_smem_attrs();
  if (e != cudaSuccess) return e;
  const long long n = lg.total_rows * 64;
  if (n > 0) k_split_phi<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(b, lg);
  return cudaGetLastError();
}

// steps x (chain step + tensor-core residual over lg.items_tc); the TMA descriptors are
// encoded once per call from lg's buffers.  steps = -1: one residual launch, no chain step.
cudaError_t launch_lg_steps_tc(const gbns_batch &b, const gbns_lg_bufs &lg, int steps, cudaStream_t s) {
  cudaError_t e = set_smem_attrs();
  if (e != cudaSuccess) return e;
  SrMaps maps;
  if (!encode_rows(&maps.w_hi, lg.W_hi, lg.total_chains, 64, 128) ||
      !encode_rows(&maps.w_lo, lg.W_lo, lg.total_chains, 64, 128) ||
      !encode_rows(&maps.phi_hi, lg.Phi_hi, lg.total_rows, 64, 128) ||
      !encode_rows(&maps.phi_lo, lg.Phi_lo, lg.total_rows, 64, 128))
    return cudaErrorInvalidValue;
  // shared memory: W tile + two Phi stages, hi and lo, nkb K blocks each (96 KB per block);
  // tensor memory: 4 accumulators of 128 columns at one CTA per SM, 2 at two CTAs per SM
  const int nkb = lg.pmax > TC_KB ? 2 : 1;
  const unsigned smem = (unsigned)nkb * 6u * SR_BOX + 1024u;
  const int per_sm = nkb == 1 ? 2 : 1, acc_stages = nkb == 1 ? 2 : 4;
  int dev = 0, sms = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
  int grid = sms * per_sm;
  if (lg.num_ctas_tc > 0 && lg.num_ctas_tc < grid) grid = lg.num_ctas_tc;
  if (grid > lg.num_items_tc) grid = lg.num_items_tc;
  const int launches = steps < 0 ? 1 : steps;
  for (int q = 0; q < launches; ++q) {
    if (steps >= 0 && (e = launch_lg_chain_step(b, lg, s)) != cudaSuccess) return e;
    if (grid > 0) {
      // programmatic serialisation: the prologue (barriers, tensor memory) overlaps the chain
      // step's tail; the kernel waits for that grid before reading its output
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3((unsigned)grid);
      cfg.blockDim = dim3(SR_THREADS);
      cfg.dynamicSmemBytes = smem;
      cfg.stream = s;
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
      attr[0].val.programmaticStreamSerializationAllowed = 1;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      if ((e = cudaLaunchKernelEx(&cfg, k_lg_resid_tc, maps, b, lg, nkb, acc_stages)) != cudaSuccess) return e;
    }
  }
  return cudaGetLastError();
}


// Launch configuration of the fused shell: clusters of lg.cluster_size CTAs over lg.items_fused.
static cudaError_t lf_config(const gbns_lg_bufs &lg, cudaStream_t s, cudaLaunchConfig_t &cfg, cudaLaunchAttribute *attr,
                             LfArgs &la) {
  const int cs = lg.cluster_size, R = lg.rows_per_cta, nkb = lg.pmax > TC_KB ? 2 : 1;
  if ((cs != 8 && cs != 16) || (R != 128 && R != 256 && R != 512) || nkb * R > 512 || lg.num_items_fused < 1 ||
      !lg.items_fused)
    return cudaErrorInvalidValue;
  const int cpc = LF_M_TILE / cs;
  // Phi slice and W tile (hi, lo), y slice, partial sums, counts; at least 1/(512/R + 1) of an
  // SM's shared memory, so that the CTAs resident on one SM never ask for more than its 512
  // tensor-memory columns (an allocation that has to wait could stall a cluster barrier)
  size_t smem = 1024 + (size_t)2 * nkb * R * 128 + (size_t)2 * nkb * 16384 + (size_t)R * 4 +
                (size_t)cs * (cpc / 4) * cpc * 8 + (size_t)cs * 4;
  const size_t per_sm = 233472, floor_bytes = per_sm / (size_t)(512 / R + 1) + 1;
  if (smem < floor_bytes) smem = floor_bytes;
  if (smem > 232448) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(k_lg_shell_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess && cs > 8)
    e = cudaFuncSetAttribute(k_lg_shell_fused, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  if (e != cudaSuccess) return e;
  cfg = cudaLaunchConfig_t{};
  cfg.gridDim = dim3((unsigned)(lg.num_items_fused * cs));
  cfg.blockDim = dim3((unsigned)(32 * cpc));
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)cs;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  la.cs = cs;
  la.rows = R;
  la.nkb = nkb;
  la.cpc = cpc;
  return cudaSuccess;
}

cudaError_t launch_lg_shell_fused(const gbns_batch &b, const gbns_lg_bufs &lg, cudaStream_t s) {
  cudaLaunchConfig_t cfg;
  cudaLaunchAttribute attr[1];
  LfArgs la;
  cudaError_t e = lf_config(lg, s, cfg, attr, la);
  if (e != cudaSuccess) return e;
  LfMaps maps;
  if (!encode_rows(&maps.phi_hi, lg.Phi_hi, lg.total_rows, 64, 128) ||
      !encode_rows(&maps.phi_lo, lg.Phi_lo, lg.total_rows, 64, 128))
    return cudaErrorInvalidValue;
  e = cudaLaunchKernelEx(&cfg, k_lg_shell_fused, maps, b, lg, la);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

// Clusters of this configuration that the device can hold at once (0: it cannot launch).
cudaError_t lg_fused_max_clusters(const gbns_lg_bufs &lg, int *out) {
  cudaLaunchConfig_t cfg;
  cudaLaunchAttribute attr[1];
  LfArgs la;
  cudaError_t e = lf_config(lg, 0, cfg, attr, la);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveClusters(out, k_lg_shell_fused, &cfg);
}

cudaError_t launch_adjoint_tc(const double *U, const double *log_w, long long M, int P, const float *Phi, const float *y,
                              int N, double log_tau, double log_sigma, double *out, double *ss, double *ry,
                              float *w_scratch, float *phi_scratch, int *status, cudaStream_t s) {
  cudaError_t e = set_smem_attrs();
  if (e == cudaSuccess) e = cudaMemsetAsync(ss, 0, sizeof(double) * M, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(ry, 0, sizeof(double) * M, s);
  if (e != cudaSuccess) return e;
  const int ld = P > TC_KB ? 64 : 32;
  if (M > 0) {
    float *w_hi = w_scratch, *w_lo = w_scratch + M * ld;
    float *p_hi = phi_scratch, *p_lo = phi_scratch + (long long)N * ld;
    const long long tot = (M + N) * (long long)ld;
    k_adj_split<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(U, M, P, Phi, N, (float)exp(log_tau), ld, w_hi, w_lo,
                                                              p_hi, p_lo);
    TcMaps maps;
    if (!encode_rows(&maps.a_hi, w_hi, M, ld, TC_M) || !encode_rows(&maps.a_lo, w_lo, M, ld, TC_M) ||
        !encode_rows(&maps.b_hi, p_hi, N, ld, TC_N) || !encode_rows(&maps.b_lo, p_lo, N, ld, TC_N))
      return cudaErrorInvalidValue;
    dim3 grid((unsigned)((M + TC_M - 1) / TC_M), (unsigned)((N + TC_N - 1) / TC_N));
    k_adj_resid_tc<<<grid, 128, (ld / TC_KB) * TC_KB_BYTES + 1024, s>>>(maps, M, P, N, y, ss, ry, status);
  }
  return launch_adjoint_reduce(log_w, M, N, log_sigma, ss, ry, out, s);
}

}  // namespace gbns

namespace {
int tc_fail(int code, const char *msg) {
  gbns::record_error(msg);
  return code;
}
}  // namespace

extern "C" {

namespace {
int fused_check(const gbns_batch *batch, const gbns_lg_bufs *lg, const char *who) {
  char msg[256];
  if (!batch || !lg || batch->num_runs <= 0 || lg->pmax < 1 || lg->pmax > 64 || !lg->Phi_hi || !lg->Phi_lo ||
      !lg->row_base || lg->total_rows < 1 || !lg->items_fused || lg->num_items_fused < 1) {
    std::snprintf(msg, sizeof msg, "%s: bad arguments (Phi_hi, Phi_lo, row_base, items_fused and 1 <= pmax <= 64 "
                  "required)", who);
    return tc_fail(-1, msg);
  }
  const int R = lg->rows_per_cta, nkb = lg->pmax > 32 ? 2 : 1;
  if ((lg->cluster_size != 8 && lg->cluster_size != 16) || (R != 128 && R != 256 && R != 512) || nkb * R > 512 ||
      lg->max_steps < 1) {
    std::snprintf(msg, sizeof msg, "%s: cluster_size must be 8 or 16, rows_per_cta 128, 256 or 512 with "
                  "rows_per_cta * ceil(pmax / 32) <= 512, max_steps >= 1", who);
    return tc_fail(-1, msg);
  }
  if (batch->gradient_guided || batch->gradient_slice) {
    std::snprintf(msg, sizeof msg, "%s: the gradient options run on the lock step (gbns_lg_steps), not the fused shell",
                  who);
    return tc_fail(-1, msg);
  }
  return 0;
}
}  // namespace

int gbns_lg_shell_fused(const gbns_batch *batch, const gbns_lg_bufs *lg, void *stream) {
  int rc = fused_check(batch, lg, "gbns_lg_shell_fused");
  if (rc) return rc;
  cudaError_t e = gbns::launch_lg_shell_fused(*batch, *lg, (cudaStream_t)stream);
  if (e != cudaSuccess) return tc_fail(-2, cudaGetErrorString(e));
  return 0;
}

int gbns_lg_fused_max_clusters(const gbns_batch *batch, const gbns_lg_bufs *lg, int *max_clusters) {
  int rc = fused_check(batch, lg, "gbns_lg_fused_max_clusters");
  if (rc) return rc;
  if (!max_clusters) return tc_fail(-1, "gbns_lg_fused_max_clusters: NULL output");
  *max_clusters = 0;
  cudaError_t e = gbns::lg_fused_max_clusters(*lg, max_clusters);
  if (e != cudaSuccess) return tc_fail(-2, cudaGetErrorString(e));
  return 0;
}

int gbns_lg_iterate(const gbns_batch *batch, const gbns_lg_bufs *lg, int num_iterations, void *stream) {
  int rc = fused_check(batch, lg, "gbns_lg_iterate");
  if (rc) return rc;
  if (num_iterations < 0) return tc_fail(-1, "gbns_lg_iterate: negative iteration count");
  for (int k = 0; k < num_iterations; ++k) {
    cudaError_t e = gbns::launch_lg_shell_fused(*batch, *lg, (cudaStream_t)stream);
    if (e == cudaSuccess) e = gbns::launch_merge(*batch, (cudaStream_t)stream);
    if (e != cudaSuccess) return tc_fail(-2, cudaGetErrorString(e));
  }
  return 0;
}

int gbns_lg_prepare_tc(const gbns_batch *batch, const gbns_lg_bufs *lg, void *stream) {
  if (!batch || !lg || batch->num_runs <= 0 || !lg->Phi_hi || !lg->Phi_lo || !lg->row_base || lg->total_rows < 1)
    return tc_fail(-1, "gbns_lg_prepare_tc: bad arguments (Phi_hi, Phi_lo, row_base and total_rows >= 1 required)");
  cudaError_t e = gbns::lg_tc_prepare(*batch, *lg, (cudaStream_t)stream);
  if (e != cudaSuccess) return tc_fail(-2, cudaGetErrorString(e));
  return 0;
}

int gbns_evidence_adjoint_tc(const double *U_dev, const double *log_w_dev, long long M, int P, const float *Phi_dev,
                             const float *y_dev, int N, double log_tau, double log_sigma, double *out_dev,
                             double *ss_scratch_dev, double *ry_scratch_dev, float *w_scratch_dev,
                             float *phi_scratch_dev, int *status_dev, void *stream) {
  if (M < 0 || M > 2147483647ll || P < 1 || P > 64 || N < 1 || !out_dev || !Phi_dev || !y_dev || !status_dev ||
      !phi_scratch_dev ||
      (M > 0 && (!U_dev || !log_w_dev || !ss_scratch_dev || !ry_scratch_dev || !w_scratch_dev)))
    return tc_fail(-1, "gbns_evidence_adjoint_tc: bad arguments (1 <= P <= 64, 0 <= M < 2^31, scratch required)");
  cudaError_t e = gbns::launch_adjoint_tc(U_dev, log_w_dev, M, P, Phi_dev, y_dev, N, log_tau, log_sigma, out_dev,
                                          ss_scratch_dev, ry_scratch_dev, w_scratch_dev, phi_scratch_dev, status_dev,
                                          (cudaStream_t)stream);
  if (e != cudaSuccess) return tc_fail(-2, cudaGetErrorString(e));
  return 0;
}

}  // extern "C"
