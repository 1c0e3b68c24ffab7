// bem_tc.cu -- the BEM product Y = B X on the tensor cores (bem_precision 3).
//
// The dense boundary matrix B (nb x nb, the double-layer operator of
// bem3d.ml:938-1047 that the reference applies as an mpidense MatMult,
// nsim.ml:3128-3140) is held as three BF16 planes, B ~ B_hi + B_mid + B_lo
// (each plane the BF16 rounding of what the previous ones leave, ~24
// significant bits together); every right-hand side x (a boundary potential)
// is split the same way when the product is formed.  The product keeps the
// six terms down to ~2^-24 of |B||x|:
//   hi.hi + hi.mid + mid.hi + hi.lo + mid.mid + lo.hi
// each a tcgen05.mma (kind::f16, BF16 operands, FP32 accumulation in TMEM),
// operands staged in shared memory by TMA (cp.async.bulk.tensor, 128-byte
// swizzle).  The K dimension (the boundary nodes the matrix sums over) is
// split over CTAs, each accumulating at most kKbPerSplit x 64 terms of every
// sum in FP32 (the hi.hi term and the five smaller terms in two separate TMEM
// accumulators); the per-split partial sums are added in FP64, in split
// order, by a second kernel.  So the FP32 accumulation error stays at the
// level of a thousand terms, not of nb.
//
// Tiles: 128 rows of B (one TMEM lane each) x NT right-hand sides (TMEM
// columns) x 64 entries of K per stage; one thread issues the TMA loads, one
// the MMAs, four warps read TMEM back.  Every mbarrier wait is bounded; on a
// timeout the kernel sets an error flag, stops issuing, waits (bounded) for
// its own MMAs, frees its TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <cstring>

#include "nmg_internal.h"

namespace nmg {
namespace {

// K entries per stage: 32 (rows of 64 bytes, 64-byte swizzle: 4-6 stages
// fit in shared memory; 0.532 ms per 128-vector film product) or, built with
// -DNMG_TC_KB=64, 64 (128-byte rows and swizzle, half as many stages; 0.568 ms)
#ifndef NMG_TC_KB
#define NMG_TC_KB 32
#endif
constexpr int kTcRows = 128;                      // rows of B per CTA (MMA M)
constexpr int kTcK = NMG_TC_KB;
static_assert(kTcK == 64 || kTcK == 32, "K block of 64 or 32 BF16 entries");
constexpr int kRowBytes = 2 * kTcK;               // one swizzle span
constexpr int kKbPerSplit = 1024 / kTcK;          // K stages accumulated in TMEM per split (1024 terms)
constexpr int kStMul = 64 / kTcK;                 // stages: twice as many with the 32-entry block
constexpr unsigned long long kTcSpinLimit = 1ull << 26;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for the given phase parity; false if it gave up (or another
// thread of the CTA already gave up).
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity, volatile int *abort_flag) {
  for (unsigned long long spins = 0; !mbar_try_wait(bar, parity); ++spins)
    if (spins > kTcSpinLimit || *abort_flag) return false;
  return true;
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y)
      : "memory");
}

// Shared-memory matrix descriptor of a K-major tile with the swizzle of its
// row length (rows of kRowBytes, groups of 8 rows 8 kRowBytes apart): start
// address, leading offset 0 (unused for these layouts), stride offset
// 8 kRowBytes, the fixed version bits (0b001 at bit 46) and the swizzle mode
// (2: 128 bytes, 4: 64 bytes).
__device__ __forceinline__ uint64_t desc_sw(uint32_t saddr) {
  constexpr uint64_t mode = kRowBytes == 128 ? 2 : 4;
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((8 * kRowBytes) >> 4) << 32) | ((uint64_t)1 << 46) |
         (mode << 61);
}

// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), BF16
// A and B (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, int accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// part[(ks * Rstride + n) * Mpad + row]: the FP32 sum over split ks of
// B[row][k] x_n[k], where plane p of the right-hand sides starts at row
// p * Rstride of tX.  Grid: (Mpad / 128, ceil(R / NT), splits); 128 threads.
template <int NT, int ST>
__global__ void __launch_bounds__(128, 1)
    k_bem_tc(const __grid_constant__ CUtensorMap tA, const __grid_constant__ CUtensorMap tX, int Mpad, int Rstride,
             int kb_total, float *__restrict__ part, int *__restrict__ err) {
  constexpr uint32_t kABytes = kTcRows * kTcK * 2, kXBytes = NT * kTcK * 2;
  constexpr uint32_t kStageBytes = 3 * (kABytes + kXBytes);
  extern __shared__ uint8_t dsm_raw[];
  __shared__ uint64_t full[ST], empty[ST], done;
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_flag, n_issued, n_consumed;
  // the six (A plane, X plane) pairs of the split product, largest first
  constexpr int kPairA[6] = {0, 0, 1, 0, 1, 2};
  constexpr int kPairX[6] = {0, 1, 0, 2, 1, 0};
  uint8_t *sm = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(dsm_raw) + 1023) & ~uintptr_t(1023));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int kb0 = blockIdx.z * kKbPerSplit;
  const int nkb = min(kb_total, kb0 + kKbPerSplit) - kb0;
  if (threadIdx.x == 0) {
    for (int s = 0; s < ST; ++s) { mbar_init(&full[s], 1); mbar_init(&empty[s], 1); }
    mbar_init(&done, 1);
    abort_flag = 0;
    n_issued = n_consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // 2 NT TMEM columns (a power of two >= 64): two 128 x NT FP32 accumulators,
  // columns [0, NT) for the hi.hi term, [NT, 2 NT) for the five smaller ones,
  // so the small terms' rounding is relative to their own (2^-8 smaller) sums
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"((uint32_t)(2 * NT)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;
  volatile int *abort_v = &abort_flag;
  auto tileA = [&](int s, int p) { return sm + (size_t)s * kStageBytes + (size_t)p * kABytes; };
  auto tileX = [&](int s, int p) { return sm + (size_t)s * kStageBytes + 3 * kABytes + (size_t)p * kXBytes; };

  if (warp == 0 && lane == 0) {   // TMA producer
    for (int i = 0; i < nkb; ++i) {
      const int s = i % ST;
      if (i >= ST && !mbar_wait(&empty[s], ((i / ST) & 1) ^ 1, abort_v)) { *abort_v = 1; break; }
      mbar_expect_tx(&full[s], kStageBytes);
      const int kx = (kb0 + i) * kTcK;
      for (int p = 0; p < 3; ++p) tma_load_2d(tileA(s, p), &tA, kx, p * Mpad + blockIdx.x * kTcRows, &full[s]);
      for (int p = 0; p < 3; ++p) tma_load_2d(tileX(s, p), &tX, kx, p * Rstride + blockIdx.y * NT, &full[s]);
      n_issued = i + 1;
    }
  } else if (warp == 1 && lane == 0) {   // MMA issuer
    constexpr uint32_t idesc = idesc_bf16(kTcRows, NT);
    for (int i = 0; i < nkb; ++i) {
      const int s = i % ST;
      if (!mbar_wait(&full[s], (i / ST) & 1, abort_v)) { *abort_v = 1; break; }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      uint64_t da[3], dx[3];
      for (int p = 0; p < 3; ++p) { da[p] = desc_sw(smem_u32(tileA(s, p))); dx[p] = desc_sw(smem_u32(tileX(s, p))); }
#pragma unroll
      for (int kk = 0; kk < kTcK / 16; ++kk)   // 16 entries (32 bytes) per MMA: +2 in the encoded address
#pragma unroll
        for (int t = 0; t < 6; ++t)
          mma_bf16(t == 0 ? tmem : tmem + NT, da[kPairA[t]] + 2 * kk, dx[kPairX[t]] + 2 * kk, idesc,
                   (i | kk | (t > 1 ? 1 : 0)) != 0);
      mma_commit(&empty[s]);   // the stage is free once these MMAs have read it
      n_consumed = i + 1;
    }
    mma_commit(&done);         // tracks every MMA issued above
  }
  __syncwarp();
  // epilogue: warp w reads TMEM lanes 32w..32w+31 (rows of this tile)
  const bool ok = mbar_wait(&done, 0, abort_v) && !*abort_v;
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (ok) {
    const int row = blockIdx.x * kTcRows + warp * 32 + lane;
    float *out = part + ((size_t)blockIdx.z * Rstride + (size_t)blockIdx.y * NT) * Mpad + row;
#pragma unroll 1
    for (int c0 = 0; c0 < NT; c0 += 32) {
      uint32_t r0[32], r1[32];
      tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, r0);
      tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(NT + c0), r1);
#pragma unroll
      for (int j = 0; j < 32; ++j)
        out[(size_t)(c0 + j) * Mpad] = (float)((double)__uint_as_float(r0[j]) + (double)__uint_as_float(r1[j]));
    }
  } else if (threadIdx.x == 0) {
    atomicOr(err, ERR_BARRIER);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (!ok && threadIdx.x == 32) {   // let the MMAs issued so far finish before the TMEM goes (bounded)
    for (unsigned long long spins = 0; !mbar_try_wait(&done, 0) && spins < kTcSpinLimit; ++spins) {
    }
  }
  if (!ok && threadIdx.x == 0) {    // and the TMA loads issued but never consumed land before the CTA exits
    for (int i = n_consumed; i < n_issued; ++i)
      for (unsigned long long spins = 0; !mbar_try_wait(&full[i % ST], (i / ST) & 1) && spins < kTcSpinLimit;
           ++spins) {
      }
  }
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)(2 * NT)));
}

// y[n * nb + row] = sum over the splits, in split order, of the FP32 partials (FP64 adds).
__global__ void k_tc_reduce(int nb, int R, int Rpad, int Mpad, int splits, const float *__restrict__ part,
                            double *__restrict__ y) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)R * nb) return;
  const int n = (int)(idx / nb), row = (int)(idx % nb);
  double s = 0.0;
  for (int k = 0; k < splits; ++k) s += (double)__ldcs(part + ((size_t)k * Rpad + n) * Mpad + row);
  y[idx] = s;
}

// Three BF16 planes of a row-major FP64 matrix (rows x cols, row stride lds)
// into planes of rows padded to rpad and columns to ldk (the pads stay zero).
__global__ void k_split3_bf16(int rows, int cols, int lds, const double *__restrict__ src, int rpad, int ldk,
                              __nv_bfloat16 *__restrict__ dst) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)rows * cols) return;
  const int r = (int)(idx / cols), c = (int)(idx % cols);
  const double v = src[(size_t)r * lds + c];
  const __nv_bfloat16 hi = __double2bfloat16(v);
  const double r1 = v - (double)__bfloat162float(hi);
  const __nv_bfloat16 mid = __double2bfloat16(r1);
  const double r2 = r1 - (double)__bfloat162float(mid);
  const __nv_bfloat16 lo = __double2bfloat16(r2);
  const size_t plane = (size_t)rpad * ldk, at = (size_t)r * ldk + c;
  dst[at] = hi;
  dst[plane + at] = mid;
  dst[2 * plane + at] = lo;
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    cudaDriverEntryPointQueryResult q;
    void *p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// 2D BF16 tensor map over rows x ldk (row-major), box kTcK x box_rows, swizzled like the tiles.
bool encode_planes(CUtensorMap *map, void *base, int ldk, int rows, int box_rows) {
  auto fn = encode_fn();
  if (!fn) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)ldk, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)ldk * 2};
  const cuuint32_t box[2] = {(cuuint32_t)kTcK, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
            kRowBytes == 128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int nt_for(int R) { return R <= 32 ? 32 : (R <= 64 ? 64 : 128); }

template <int NT, int ST>
size_t tc_smem() {
  return (size_t)ST * 3 * (kTcRows + NT) * kTcK * 2 + 1024;
}

}  // namespace

// Planes of the handle's FP64 BEM and the tensor map over them.
int bem_tc_setup(nmg_handle *h, std::string &err) {
  Mesh &M = h->mesh;
  TcState &T = h->tc;
  const int nb = M.nb;
  T.Mpad = (nb + kTcRows - 1) / kTcRows * kTcRows;
  T.ldk = (nb + 63) / 64 * 64;   // a whole number of K blocks of either size
  const size_t plane = (size_t)T.Mpad * T.ldk;
  NMG_CUDA_TRY(T.bplanes.alloc(3 * plane), "alloc BF16 BEM planes");
  NMG_CUDA_TRY(cudaMemsetAsync(T.bplanes.p, 0, sizeof(uint16_t) * 3 * plane, h->stream), "zero BF16 planes");
  const long long n = (long long)nb * nb;
  k_split3_bf16<<<(unsigned)((n + 255) / 256), 256, 0, h->stream>>>(
      nb, nb, M.ld, M.bem, T.Mpad, T.ldk, reinterpret_cast<__nv_bfloat16 *>(T.bplanes.p));
  ++h->launches;
  NMG_CUDA_TRY(cudaGetLastError(), "split BEM planes");
  static_assert(sizeof(CUtensorMap) == sizeof(T.mapA), "tensor map storage");
  if (!encode_planes(reinterpret_cast<CUtensorMap *>(T.mapA), T.bplanes.p, T.ldk, 3 * T.Mpad, kTcRows)) {
    err = "bem_tc_setup: cuTensorMapEncodeTiled failed for the BEM planes";
    return 100;
  }
  NMG_CUDA_TRY(cudaStreamSynchronize(h->stream), "BF16 BEM planes");
  return 0;
}

// Room for R right-hand sides: X planes (zero pads), partials, the X tensor map.
static int tc_reserve(nmg_handle *h, int R, std::string &err) {
  TcState &T = h->tc;
  const int NT = nt_for(R);
  const int Rpad = (R + NT - 1) / NT * NT;
  if (T.xplanes.p && Rpad <= T.Rcap && NT == T.nt) return 0;
  if (T.xplanes.p && Rpad <= T.Rcap && (T.Rcap % NT) == 0) {   // the buffers fit: only the tile width changes
    T.nt = NT;
    if (!encode_planes(reinterpret_cast<CUtensorMap *>(T.mapX), T.xplanes.p, T.ldk, 3 * T.Rcap, NT)) {
      err = "bem_tc: cuTensorMapEncodeTiled failed for the x planes";
      return 100;
    }
    return 0;
  }
  T.nt = NT;
  T.Rcap = Rpad;
  const size_t plane = (size_t)Rpad * T.ldk;
  NMG_CUDA_TRY(T.xplanes.alloc(3 * plane), "alloc BF16 x planes");
  NMG_CUDA_TRY(cudaMemsetAsync(T.xplanes.p, 0, sizeof(uint16_t) * 3 * plane, h->stream), "zero x planes");
  const int splits = (T.ldk / kTcK + kKbPerSplit - 1) / kKbPerSplit;
  NMG_CUDA_TRY(T.part.alloc((size_t)splits * Rpad * T.Mpad), "alloc tensor-core partials");
  if (!encode_planes(reinterpret_cast<CUtensorMap *>(T.mapX), T.xplanes.p, T.ldk, 3 * Rpad, NT)) {
    err = "bem_tc: cuTensorMapEncodeTiled failed for the x planes";
    return 100;
  }
  return 0;
}

// Y = B X for R right-hand sides (member-major: x_n at x + n * nb).
int bem_tc(nmg_handle *h, const double *x, double *y, int R) {
  Mesh &M = h->mesh;
  TcState &T = h->tc;
  const int nb = M.nb;
  std::string err;
  if (!T.bplanes.p || tc_reserve(h, R, err)) {
    h->last_error = err.empty() ? "bem_tc: tensor-core planes not set up" : err;
    return 100;
  }
  const int NT = T.nt, Rpad = T.Rcap;   // Rpad: the planes' row stride (rows >= R are never read back)
  const long long n = (long long)R * nb;
  k_split3_bf16<<<(unsigned)((n + 255) / 256), 256, 0, h->stream>>>(
      R, nb, nb, x, Rpad, T.ldk, reinterpret_cast<__nv_bfloat16 *>(T.xplanes.p));
  ++h->launches;
  const int kb_total = T.ldk / kTcK;
  const int splits = (kb_total + kKbPerSplit - 1) / kKbPerSplit;
  const dim3 grid(T.Mpad / kTcRows, (R + NT - 1) / NT, splits);
  const CUtensorMap &mA = *reinterpret_cast<const CUtensorMap *>(T.mapA);
  const CUtensorMap &mX = *reinterpret_cast<const CUtensorMap *>(T.mapX);
  {
    NMG_PROF_BEGIN(h, 0);
    if (NT == 32) {
      const size_t sm = tc_smem<32, 3 * kStMul>();
      cudaFuncSetAttribute(k_bem_tc<32, 3 * kStMul>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      k_bem_tc<32, 3 * kStMul><<<grid, 128, sm, h->stream>>>(mA, mX, T.Mpad, Rpad, kb_total, T.part, h->ws.err);
    } else if (NT == 64) {
      const size_t sm = tc_smem<64, 3 * kStMul>();
      cudaFuncSetAttribute(k_bem_tc<64, 3 * kStMul>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      k_bem_tc<64, 3 * kStMul><<<grid, 128, sm, h->stream>>>(mA, mX, T.Mpad, Rpad, kb_total, T.part, h->ws.err);
    } else {
      const size_t sm = tc_smem<128, 2 * kStMul>();
      cudaFuncSetAttribute(k_bem_tc<128, 2 * kStMul>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      k_bem_tc<128, 2 * kStMul><<<grid, 128, sm, h->stream>>>(mA, mX, T.Mpad, Rpad, kb_total, T.part, h->ws.err);
    }
    ++h->launches;
    NMG_PROF_END(h);
  }
  k_tc_reduce<<<(unsigned)((n + 255) / 256), 256, 0, h->stream>>>(nb, R, Rpad, T.Mpad, splits, T.part, y);
  ++h->launches;
  if (cudaGetLastError() != cudaSuccess) {
    h->last_error = "bem_tc: launch failed";
    return 100;
  }
  return 0;
}

}  // namespace nmg
