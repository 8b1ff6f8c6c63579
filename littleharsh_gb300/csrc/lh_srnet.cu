// lh_srnet.cu -- BF16 tensor-core kernels of the super-resolution network
// that lifts a coarse-grid field onto the fine grid (the learned warm start).
//
// The reference has no counterpart: its only initial conditions are a restart
// file or a parabolic profile (start.f90:1488-1784).
//
// Activations are channels-last volumes [y][z][x][c] in bf16 with c = 16 or
// 32; x and z are periodic (the Fourier directions of the channel), y is
// zero-padded.  A 3x3x3 convolution is an implicit GEMM: rows = voxels,
// columns = output channels, reduction = 27 taps x input channels, computed
// with mma.sync m16n8k16 (bf16 in, fp32 accumulate).  A CTA stages a tile of
// 8 z-rows x 32 x-voxels of one y level plus its halo (3 y levels x 10 z-rows
// x 34 x-voxels) in shared memory with cp.async; the weights of the layer
// stay in shared memory while the persistent CTA walks over tiles.  Fragments
// come from shared memory with ldmatrix (the tap shift is just a different
// row address).  Rows are padded by 16 bytes so the 8 row addresses of an
// ldmatrix fall in distinct bank groups.
//
// Backward:
//   data gradient = the forward kernel run on the output gradient with the
//     taps mirrored and the channel roles swapped (lh_sr_flip_weights);
//   weight gradient: rows = output channels, columns = input channels,
//     reduction = voxels, one warp per 3 taps, accumulated in registers over
//     all tiles of the persistent CTA and added to the fp32 gradient once.
// The tcgen05 forms of the forward convolution and the weight gradient follow
// the mma.sync kernels below; the network uses them by default.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "lh_internal.h"
#include "lh_srnet.h"
#include "littleharsh.h"

namespace lh {
namespace sr {

constexpr int TX = 32;            // x-voxels per tile (two m16 tiles)
constexpr int TZ = 8;             // z-rows per tile (one warp each in the forward kernel)
constexpr int HX = TX + 2, HZ = TZ + 2;
constexpr int HROWS = 3 * HZ * HX;  // staged input rows (voxels) per tile

struct Vol {
  int X, Y, Z;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void cp_async16(void* dst, const void* src, bool valid) {
  // src-size 0 fills the 16 bytes with zeros and reads nothing
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(smem_u32(dst)), "l"(src),
               "r"(valid ? 16 : 0));
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_u32(p)));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t (&r)[4], const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_u32(p)));
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Stage the input halo of tile (y, z0, x0) into sIn: rows [dy][zz][xx], each C
// channels, row stride C + 8 elements.
template <int C>
__device__ __forceinline__ void stage_halo(__nv_bfloat16* sIn, const __nv_bfloat16* __restrict__ in, const Vol v,
                                           int y, int z0, int x0) {
  constexpr int CH = C / 8;  // 16-byte chunks per row
  constexpr int RS = C + 8;
  for (int c = threadIdx.x; c < HROWS * CH; c += blockDim.x) {
    const int row = c / CH, part = c - row * CH;
    const int xx = row % HX, zz = (row / HX) % HZ, dy = row / (HX * HZ);
    const int gy = y + dy - 1;
    const bool ok = gy >= 0 && gy < v.Y;
    const int gz = (z0 + zz - 1 + v.Z) % v.Z, gx = (x0 + xx - 1 + v.X) % v.X;
    const size_t vox = ok ? ((size_t)gy * v.Z + gz) * v.X + gx : 0;
    cp_async16(sIn + (size_t)row * RS + part * 8, in + vox * C + part * 8, ok);
  }
}

enum : int { EPI_RELU = 1, EPI_RES = 2, EPI_GATE = 4, EPI_BIAS = 8 };

template <typename T> __device__ __forceinline__ void store2(T* p, float a, float b);
template <> __device__ __forceinline__ void store2<float>(float* p, float a, float b) {
  *reinterpret_cast<float2*>(p) = make_float2(a, b);
}
template <> __device__ __forceinline__ void store2<__nv_bfloat16>(__nv_bfloat16* p, float a, float b) {
  *reinterpret_cast<__nv_bfloat162*>(p) = __floats2bfloat162_rn(a, b);
}

// out[v][co] = epi( sum_tap sum_ci W[tap][co][ci] in[nbr(v, tap)][ci] )
// epi: + bias, ReLU, zero where gate <= 0, + res (in this order, each optional)
template <int CIN, int COUT, typename OutT>
__global__ void __launch_bounds__(TZ * 32, 1)
    k_conv_fwd(const __nv_bfloat16* __restrict__ in, const __nv_bfloat16* __restrict__ w,
               const float* __restrict__ bias, OutT* __restrict__ out, const __nv_bfloat16* __restrict__ res,
               const __nv_bfloat16* __restrict__ gate, int epi, Vol v) {
  constexpr int RSI = CIN + 8, RSW = CIN + 8;
  constexpr int NT = COUT / 8;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __nv_bfloat16* sW = reinterpret_cast<__nv_bfloat16*>(smem_raw);
  __nv_bfloat16* sIn = sW + 27 * COUT * RSW;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

  // weights [27][COUT][CIN] -> rows of RSW
  for (int c = threadIdx.x; c < 27 * COUT * (CIN / 8); c += blockDim.x) {
    const int row = c / (CIN / 8), part = c - row * (CIN / 8);
    cp_async16(sW + (size_t)row * RSW + part * 8, w + (size_t)row * CIN + part * 8, true);
  }
  const int ntx = v.X / TX, ntz = v.Z / TZ;
  const int ntiles = v.Y * ntz * ntx;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int xt = tile % ntx, rest = tile / ntx, zt = rest % ntz, y = rest / ntz;
    const int x0 = xt * TX, z0 = zt * TZ;
    __syncthreads();  // the previous tile's fragments have been read
    stage_halo<CIN>(sIn, in, v, y, z0, x0);
    cp_async_wait_all();
    __syncthreads();

    float acc[2][NT][4];
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
      for (int j = 0; j < NT; ++j)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[mt][j][q] = 0.f;

    const int zr = warp;
    const int arow = (lane & 7) + ((lane >> 3) & 1) * 8;  // A: row within the m16 tile
    const int acol = (lane >> 4) * 8;                      // A: k offset
    const int bn = (lane >> 4) * 8 + (lane & 7);           // B: n within a pair of n8 tiles
    const int bk = ((lane >> 3) & 1) * 8;                  // B: k offset
#pragma unroll 1
    for (int tap = 0; tap < 27; ++tap) {
      const int dy = tap / 9, dz = (tap / 3) % 3, dx = tap % 3;
      const __nv_bfloat16* rowbase = sIn + (size_t)((dy * HZ + zr + dz) * HX + dx) * RSI;
      const __nv_bfloat16* wbase = sW + (size_t)tap * COUT * RSW;
#pragma unroll
      for (int kc = 0; kc < CIN / 16; ++kc) {
        uint32_t a[2][4];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) ldsm_x4(a[mt], rowbase + (size_t)(mt * 16 + arow) * RSI + kc * 16 + acol);
#pragma unroll
        for (int j = 0; j < NT; j += 2) {
          uint32_t b[4];
          ldsm_x4(b, wbase + (size_t)(j * 8 + bn) * RSW + kc * 16 + bk);
#pragma unroll
          for (int mt = 0; mt < 2; ++mt) {
            mma_bf16(acc[mt][j], a[mt], b[0], b[1]);
            mma_bf16(acc[mt][j + 1], a[mt], b[2], b[3]);
          }
        }
      }
    }
    // epilogue
    const int g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
      for (int half = 0; half < 2; ++half) {
        const int x = x0 + mt * 16 + g + half * 8;
        const size_t vox = ((size_t)y * v.Z + z0 + zr) * v.X + x;
#pragma unroll
        for (int j = 0; j < NT; ++j) {
          const int n = j * 8 + 2 * t;
          float r0 = acc[mt][j][2 * half], r1 = acc[mt][j][2 * half + 1];
          if (epi & EPI_BIAS) { r0 += bias[n]; r1 += bias[n + 1]; }
          if (epi & EPI_RELU) { r0 = fmaxf(r0, 0.f); r1 = fmaxf(r1, 0.f); }
          if (epi & EPI_GATE) {
            const __nv_bfloat162 gv = *reinterpret_cast<const __nv_bfloat162*>(gate + vox * COUT + n);
            if (!(__low2float(gv) > 0.f)) r0 = 0.f;
            if (!(__high2float(gv) > 0.f)) r1 = 0.f;
          }
          if (epi & EPI_RES) {
            const __nv_bfloat162 rv = *reinterpret_cast<const __nv_bfloat162*>(res + vox * COUT + n);
            r0 += __low2float(rv);
            r1 += __high2float(rv);
          }
          store2<OutT>(out + vox * COUT + n, r0, r1);
        }
      }
  }
  cp_async_wait_all();  // a CTA without a tile still drains its weight copies
}

// dW[tap][co][ci] += sum_v dout[v][co] in[nbr(v, tap)][ci]; db[co] += sum_v dout[v][co].
// Warp w owns taps 3w .. 3w+2 (9 warps); M = output channels (m16 tiles),
// N = input channels (n8 tiles), K = the tile's voxels, 16 at a time.
constexpr int WG_WARPS = 9;
template <int CIN, int COUT>
__global__ void __launch_bounds__(WG_WARPS * 32, 1)
    k_conv_wgrad(const __nv_bfloat16* __restrict__ in, const __nv_bfloat16* __restrict__ dout,
                 float* __restrict__ dw, float* __restrict__ db, Vol v) {
  constexpr int RSI = CIN + 8, RSD = COUT + 8;
  constexpr int MT = COUT / 16, NT = CIN / 8;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __nv_bfloat16* sIn = reinterpret_cast<__nv_bfloat16*>(smem_raw);
  __nv_bfloat16* sD = sIn + (size_t)HROWS * RSI;
  float* sBias = reinterpret_cast<float*>(sD + (size_t)TZ * TX * RSD);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < COUT; i += blockDim.x) sBias[i] = 0.f;

  float acc[3][MT][NT][4];
#pragma unroll
  for (int q = 0; q < 3; ++q)
#pragma unroll
    for (int m = 0; m < MT; ++m)
#pragma unroll
      for (int j = 0; j < NT; ++j)
#pragma unroll
        for (int e = 0; e < 4; ++e) acc[q][m][j][e] = 0.f;
  float bacc = 0.f;  // thread < COUT: its channel's bias gradient

  const int ntx = v.X / TX, ntz = v.Z / TZ;
  const int ntiles = v.Y * ntz * ntx;
  // ldmatrix.trans row addresses: matrix q = lane / 8, row r = lane % 8
  const int qd = lane >> 3, r8 = lane & 7;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int xt = tile % ntx, rest = tile / ntx, zt = rest % ntz, y = rest / ntz;
    const int x0 = xt * TX, z0 = zt * TZ;
    __syncthreads();
    stage_halo<CIN>(sIn, in, v, y, z0, x0);
    for (int c = threadIdx.x; c < TZ * TX * (COUT / 8); c += blockDim.x) {
      const int row = c / (COUT / 8), part = c - row * (COUT / 8);
      const int xx = row % TX, zz = row / TX;
      const size_t vox = ((size_t)y * v.Z + z0 + zz) * v.X + x0 + xx;
      cp_async16(sD + (size_t)row * RSD + part * 8, dout + vox * COUT + part * 8, true);
    }
    cp_async_wait_all();
    __syncthreads();
    if (threadIdx.x < COUT) {
      float s = 0.f;
      for (int r = 0; r < TZ * TX; ++r) s += __bfloat162float(sD[(size_t)r * RSD + threadIdx.x]);
      bacc += s;
    }
#pragma unroll 1
    for (int ks = 0; ks < TZ * 2; ++ks) {
      const int zr = ks >> 1, xh = (ks & 1) * 16;
      // A = dout^T: stored rows = voxels (k), columns = channels (m)
      uint32_t a[MT][4];
#pragma unroll
      for (int m = 0; m < MT; ++m) {
        const int vrow = zr * TX + xh + (qd >> 1) * 8 + r8;
        ldsm_x4_t(a[m], sD + (size_t)vrow * RSD + m * 16 + (qd & 1) * 8);
      }
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        const int tap = warp * 3 + q;
        const int dy = tap / 9, dz = (tap / 3) % 3, dx = tap % 3;
        const int hrow = (dy * HZ + zr + dz) * HX + dx + xh + (qd & 1) * 8 + r8;
#pragma unroll
        for (int j = 0; j < NT; j += 2) {
          uint32_t b[4];
          ldsm_x4_t(b, sIn + (size_t)hrow * RSI + (j + (qd >> 1)) * 8);
#pragma unroll
          for (int m = 0; m < MT; ++m) {
            mma_bf16(acc[q][m][j], a[m], b[0], b[1]);
            mma_bf16(acc[q][m][j + 1], a[m], b[2], b[3]);
          }
        }
      }
    }
  }
  cp_async_wait_all();
  const int g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    const int tap = warp * 3 + q;
#pragma unroll
    for (int m = 0; m < MT; ++m)
#pragma unroll
      for (int j = 0; j < NT; ++j)
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int co = m * 16 + g + (e >> 1) * 8, ci = j * 8 + 2 * t + (e & 1);
          atomicAdd(dw + ((size_t)tap * COUT + co) * CIN + ci, acc[q][m][j][e]);
        }
  }
  if (threadIdx.x < COUT) atomicAdd(db + threadIdx.x, bacc);
}

// wt[tap'][ci][co] = w[26 - tap'][co][ci]: the data gradient of a convolution
// is the convolution of the output gradient with the mirrored, transposed taps
__global__ void k_flip_weights(const __nv_bfloat16* __restrict__ w, __nv_bfloat16* __restrict__ wt, int cin,
                               int cout) {
  const int n = 27 * cin * cout;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int co = i % cout, rest = i / cout, ci = rest % cin, tap = rest / cin;
    wt[i] = w[((size_t)(26 - tap) * cout + co) * cin + ci];
  }
}

// Loss of one sample: pred = base + corr (channels 0..2 of the network's fp32
// output, 16 channels per voxel), L = sum (pred - target)^2 / (3 nvox);
// dcorr = dL/dcorr in bf16 with channels 3..15 zero.  `loss` gets L added.
__global__ void k_mse(const float* __restrict__ corr, const float* __restrict__ base,
                      const float* __restrict__ target, __nv_bfloat16* __restrict__ dcorr, double* __restrict__ loss,
                      long long nvox, float scale) {
  __shared__ float red[32];
  float s = 0.f;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nvox; v += (long long)gridDim.x * blockDim.x) {
    float d[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      d[c] = base[v * 3 + c] + corr[v * 16 + c] - target[v * 3 + c];
      s += d[c] * d[c];
    }
    const __nv_bfloat162 o0 = __floats2bfloat162_rn(scale * 2.f * d[0], scale * 2.f * d[1]);
    const __nv_bfloat162 o1 = __floats2bfloat162_rn(scale * 2.f * d[2], 0.f);
    uint4 w0;
    w0.x = *reinterpret_cast<const uint32_t*>(&o0);
    w0.y = *reinterpret_cast<const uint32_t*>(&o1);
    w0.z = 0u;
    w0.w = 0u;
    uint4* dst = reinterpret_cast<uint4*>(dcorr + v * 16);
    dst[0] = w0;
    dst[1] = make_uint4(0u, 0u, 0u, 0u);
  }
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.f;
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if (threadIdx.x == 0) atomicAdd(loss, (double)s * (double)scale);
  }
}

// AdamW on fp32 master parameters; the bf16 copy the convolutions read is
// refreshed in the same pass.  bc1/bc2 are the bias corrections 1 - beta^t.
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, __nv_bfloat16* __restrict__ pb, int n, float lr, float b1, float b2,
                       float eps, float wd, float bc1, float bc2) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float mh = mi / bc1, vh = vi / bc2;
    const float pi = p[i] * (1.f - lr * wd) - lr * mh / (sqrtf(vh) + eps);
    p[i] = pi;
    if (pb) pb[i] = __float2bfloat16_rn(pi);
  }
}

// ---- tcgen05 forward convolution ------------------------------------------------
//
// The same convolution on the 5th-generation tensor cores.  A tile is 32
// x-voxels x 8 z-rows of one y level (M = 256 as two M = 128 halves of 16
// x-voxels, fp32 accumulators of Cout columns in TMEM).  Its work runs as three
// stages, one per y offset dy of the taps.  A stage's input is the dy level's
// halo, 34 x-voxels x 10 z-rows, held in shared memory as 16-byte rows
// [k chunk][x][z] (no-swizzle K-major core matrices of 8 rows x 16 bytes),
// x columns 11 rows apart (one row of padding spreads the copies over the
// banks).  With z fastest, a core matrix is 8 consecutive z of one x, and
// consecutive core matrices along M are consecutive x, 11 rows apart; the A
// operand of tap (dz, dx) is the same layout started dz + 11 dx rows on, so the
// nine taps of a stage read one halo copy through their descriptors' start
// addresses and nothing is copied twice.
//
// The CTA is warp-specialised, its roles ordered only by mbarriers:
//   warps 0-3 (producers) fetch halos into a ring of six buffers with 16-byte
//     loads into registers and 16-byte shared stores (cp.async with a zero-fill
//     size measured slower: its copies were not coalesced, about 32 L2 sectors
//     and 38 shared wavefronts per warp instruction against 16 and 4); each
//     thread fences its stores for the tensor core and arrives on the buffer's
//     `full` barrier (128 arrivals); a buffer is refilled after the `empty`
//     barrier says the MMAs that read it completed;
//   warp 8 (one thread) waits on `full`, issues the stage's 9 taps x Cin/16 x 2
//     tcgen05.mma (K = 16 channels, bf16 operands from shared memory) into the
//     tile's accumulator set and commits them to `empty` (and, after a tile's
//     last stage, to the set's `acc_full`);
//   warps 4-7 (epilogue) wait on `acc_full`, read TMEM lanes 32 (w mod 4) of
//     both halves with tcgen05.ld, apply bias / ReLU / gate / residual, store,
//     and arrive on `acc_empty`, which frees the set for the tile after next.
// Two accumulator sets (128 TMEM columns) let the epilogue of one tile run
// under the MMAs of the next.  Every wait is bounded; a wait that runs out
// raises a shared abort flag that ends every role's loop, and the kernel
// reports it through its error word after draining its copies and MMAs.
constexpr int TC_TZ = 8;                     // z rows per tile
constexpr int TC_ZR = TC_TZ + 2;             // halo z rows
constexpr int TC_XR = TX + 2;                // halo x voxels
constexpr int TC_HALO = TC_ZR * TC_XR;       // voxel rows of one k chunk of a halo
constexpr int TC_XP = TC_ZR + 1;             // x pitch in 16-byte rows: odd, so a warp's copies spread over all banks
constexpr int TC_KP = TC_XR * TC_XP;         // k-chunk pitch in 16-byte rows
constexpr int TC_NBUF = 6;                   // halo ring (4: 218 us, 6: 203 us, 8: 201 us on 130x96x96)
constexpr int TC_PRODUCERS = 128;            // warps 0-3
constexpr int TC_THREADS = 288;              // + epilogue warps 4-7 + MMA warp 8
constexpr int TC_MMA_WARP = 8;
constexpr unsigned kTcSpinLimit = 1u << 20;  // bound of every mbarrier wait

__device__ __forceinline__ uint64_t tc_smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  // start address, leading (K) and stride (M/N) byte offsets in 16-byte units, descriptor version 1,
  // base offset 0, no swizzle
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
__host__ __device__ constexpr uint32_t tc_idesc(int m, int n) {
  // kind::f16: D f32 (bits 4-5 = 1), A bf16 (bits 7-9 = 1), B bf16 (bits 10-12 = 1), both K-major,
  // N >> 3 at bits 17-22, M >> 4 at bits 24-28
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

// bounded wait for the phase of parity `parity` of an mbarrier; gives up early once *abort is set; false if
// the phase did not complete (and then raises *abort)
__device__ __forceinline__ bool tc_wait(uint64_t* bar, uint32_t parity, volatile int* abort) {
  uint32_t done = 0;
  for (unsigned it = 0; it < kTcSpinLimit && !done; ++it) {
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity));
    if (!done && (it & 63) == 63 && *abort) break;
  }
  if (!done) *abort = 1;
  return done != 0;
}
__device__ __forceinline__ void tc_arrive(uint64_t* bar) {
  asm volatile("{\n.reg .b64 st;\nmbarrier.arrive.shared::cta.b64 st, [%0];\n}\n" ::"r"(smem_u32(bar)) : "memory");
}

template <int CIN, int COUT, typename OutT>
__global__ void __launch_bounds__(TC_THREADS, 1)
    k_conv_fwd_tc(const __nv_bfloat16* __restrict__ in, const __nv_bfloat16* __restrict__ w,
                  const float* __restrict__ bias, OutT* __restrict__ out, const __nv_bfloat16* __restrict__ res,
                  const __nv_bfloat16* __restrict__ gate, int epi, Vol v, int* __restrict__ err) {
  constexpr int KC = CIN / 8;                       // 16-byte chunks (core-matrix columns) per voxel row
  constexpr uint32_t A_LBO = TC_KP * 16;            // next k chunk of a halo
  constexpr uint32_t A_SBO = TC_XP * 16;            // next 8 rows along M = next x
  constexpr uint32_t B_LBO = COUT * 16;             // next k chunk of a tap's weights
  constexpr int BUF = KC * TC_KP;                   // 16-byte rows per halo buffer
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint4* sA = reinterpret_cast<uint4*>(smem_raw);   // [TC_NBUF][KC][TC_XR (pitch TC_XP)][TC_ZR]
  uint4* sB = sA + (size_t)TC_NBUF * BUF;           // [27][KC][COUT]
  uint64_t* full = reinterpret_cast<uint64_t*>(sB + (size_t)27 * KC * COUT);
  uint64_t* empty = full + TC_NBUF;
  uint64_t* acc_full = empty + TC_NBUF;
  uint64_t* acc_empty = acc_full + 2;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(acc_empty + 2);
  volatile int* abort = reinterpret_cast<volatile int*>(tslot + 1);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

  for (int c = threadIdx.x; c < 27 * COUT * KC; c += blockDim.x) {  // weights -> [27][KC][COUT] rows
    const int kc = c % KC, n = (c / KC) % COUT, tap = c / (KC * COUT);
    cp_async16(sB + ((size_t)tap * KC + kc) * COUT + n, w + ((size_t)tap * COUT + n) * CIN + kc * 8, true);
  }
  asm volatile("cp.async.commit_group;\n" ::: "memory");
  if (threadIdx.x == 0) {
    for (int b = 0; b < TC_NBUF; ++b) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(full + b)), "r"(TC_PRODUCERS));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(empty + b)));
    }
    for (int a = 0; a < 2; ++a) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(acc_full + a)));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 4;\n" ::"r"(smem_u32(acc_empty + a)));
    }
    *abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == TC_MMA_WARP) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 128;\n" ::"r"(smem_u32(tslot)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");           // this thread's weight copies
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");    // -> visible to the tensor core
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = *tslot;

  const int ntx = v.X / TX, ntz = v.Z / TC_TZ;
  const int ntiles = v.Y * ntz * ntx;
  const int my_tiles = blockIdx.x < ntiles ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  const int nstages = 3 * my_tiles;

  if (warp < 4) {
    // ---- producers: stage st = (tile blockIdx.x + (st / 3) gridDim.x, dy = st % 3) into buffer st % NBUF:
    // rows [k chunk][x + 1][z + 1], x = -1 .. 32, z = -1 .. 8, periodic in x and z, zero outside y.  16-byte
    // loads into registers (a warp's loads cover contiguous voxels), then 16-byte shared stores; the buffer is
    // handed over as soon as its stores are done.
    const int p = threadIdx.x;
    constexpr int CH = TC_HALO * KC, PT = (CH + TC_PRODUCERS - 1) / TC_PRODUCERS;
    for (int s = 0; s < nstages; ++s) {
      if (s >= TC_NBUF && !tc_wait(empty + s % TC_NBUF, (uint32_t)((s / TC_NBUF - 1) & 1), abort)) break;
      const int tile = blockIdx.x + (s / 3) * gridDim.x, dy = s % 3;
      const int xt = tile % ntx, rest = tile / ntx, zt = rest % ntz, y = rest / ntz;
      const int x0 = xt * TX, z0 = zt * TC_TZ;
      const int gy = y + dy - 1;
      const bool ok = gy >= 0 && gy < v.Y;
      uint4* buf = sA + (size_t)(s % TC_NBUF) * BUF;
      uint4 r[PT];
      int row[PT];
#pragma unroll
      for (int i = 0; i < PT; ++i) {
        const int c = p + i * TC_PRODUCERS;
        r[i] = make_uint4(0u, 0u, 0u, 0u);
        row[i] = -1;
        if (c < CH) {
          const int kc = c % KC, u = c / KC;
          const int xh = u % TC_XR, zz = u / TC_XR;
          int gz = z0 + zz - 1, gx = x0 + xh - 1;
          gz = gz < 0 ? gz + v.Z : (gz >= v.Z ? gz - v.Z : gz);
          gx = gx < 0 ? gx + v.X : (gx >= v.X ? gx - v.X : gx);
          row[i] = kc * TC_KP + xh * TC_XP + zz;
          if (ok) r[i] = __ldg(reinterpret_cast<const uint4*>(in + (((size_t)gy * v.Z + gz) * v.X + gx) * CIN + kc * 8));
        }
      }
#pragma unroll
      for (int i = 0; i < PT; ++i)
        if (row[i] >= 0) buf[row[i]] = r[i];
      asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
      tc_arrive(full + s % TC_NBUF);
    }
  } else if (warp == TC_MMA_WARP) {
    // ---- MMA issue: one thread
    if (lane == 0) {
      const uint32_t idesc = tc_idesc(128, COUT);
      const uint64_t a_desc0 = tc_smem_desc(smem_u32(sA), A_LBO, A_SBO);
      const uint64_t b_desc0 = tc_smem_desc(smem_u32(sB), B_LBO, 128);
      int issued = 0;
      for (int s = 0; s < nstages; ++s) {
        const int dy = s % 3, ti = s / 3, acc = ti & 1;
        // the epilogue of tile ti - 2 has read this accumulator set
        if (dy == 0 && ti >= 2 && !tc_wait(acc_empty + acc, (uint32_t)((ti / 2 - 1) & 1), abort)) break;
        if (!tc_wait(full + s % TC_NBUF, (uint32_t)((s / TC_NBUF) & 1), abort)) break;
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        const uint64_t a_desc = a_desc0 + (uint64_t)((s % TC_NBUF) * BUF);  // start address in 16-byte units
        const uint32_t d_base = tmem + (uint32_t)(acc * 64);
#pragma unroll
        for (int t = 0; t < 9; ++t) {
          const int dz = t / 3, dx = t % 3;
#pragma unroll
          for (int ks = 0; ks < CIN / 16; ++ks) {
            const uint64_t bd = b_desc0 + (uint64_t)((dy * 9 + t) * KC * COUT + ks * 2 * COUT);
            const uint32_t accum = (dy > 0 || t > 0 || ks > 0) ? 1u : 0u;
#pragma unroll
            for (int h = 0; h < 2; ++h) {  // x-voxels 16h .. 16h+15 of the tile
              const uint64_t ad = a_desc + (uint64_t)(2 * ks * TC_KP + (16 * h + dx) * TC_XP + dz);
              asm volatile(
                  "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                  "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_base + (uint32_t)(h * 32)),
                  "l"(ad), "l"(bd), "r"(idesc), "r"(accum));
            }
          }
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
            smem_u32(empty + s % TC_NBUF)));
        if (dy == 2)
          asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
              smem_u32(acc_full + acc)));
        issued = s + 1;
      }
      // every MMA issued has completed before the accumulators can be freed (the last commit tracks them all)
      if (issued > 0) {
        const int q = issued - 1;
        volatile int no_abort = 0;
        tc_wait(empty + q % TC_NBUF, (uint32_t)((q / TC_NBUF) & 1), &no_abort);
        if (no_abort) *abort = 1;
      }
    }
    __syncwarp();
  } else {
    // ---- epilogue: warp 4 + g reads TMEM lanes 32 g .. 32 g + 31 of both halves; lane m of half h is the
    // voxel x = 16 h + m / 8, z = m mod 8 of the tile
    const int g = warp & 3;
    for (int ti = 0; ti < my_tiles; ++ti) {
      const int acc = ti & 1;
      if (!tc_wait(acc_full + acc, (uint32_t)((ti / 2) & 1), abort)) break;
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      const int tile = blockIdx.x + ti * gridDim.x;
      const int xt = tile % ntx, rest = tile / ntx, zt = rest % ntz, y = rest / ntz;
      const int m = g * 32 + lane;
#pragma unroll 1
      for (int h = 0; h < 2; ++h) {
        uint32_t r[32];
        const uint32_t taddr = tmem + ((uint32_t)(g * 32) << 16) + (uint32_t)(acc * 64 + h * 32);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
            "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
              "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
              "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
              "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
        const size_t vox = ((size_t)y * v.Z + zt * TC_TZ + (m & 7)) * v.X + xt * TX + 16 * h + (m >> 3);
        // the voxel's COUT outputs: bias, ReLU, gate, residual in that order; gate, residual and output move
        // 16 bytes at a time (the entry point requires 16-byte aligned tensors)
        float o[COUT];
#pragma unroll
        for (int n = 0; n < COUT; ++n) {
          o[n] = __uint_as_float(r[n]);
          if (epi & EPI_BIAS) o[n] += bias[n];
          if (epi & EPI_RELU) o[n] = fmaxf(o[n], 0.f);
        }
        if (epi & EPI_GATE) {
          const uint4* gp = reinterpret_cast<const uint4*>(gate + vox * COUT);
#pragma unroll
          for (int q = 0; q < COUT / 8; ++q) {
            const uint4 gv = gp[q];
            const uint32_t gw[4] = {gv.x, gv.y, gv.z, gv.w};
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              const __nv_bfloat162 g2 = *reinterpret_cast<const __nv_bfloat162*>(&gw[e]);
              if (!(__low2float(g2) > 0.f)) o[8 * q + 2 * e] = 0.f;
              if (!(__high2float(g2) > 0.f)) o[8 * q + 2 * e + 1] = 0.f;
            }
          }
        }
        if (epi & EPI_RES) {
          const uint4* rp = reinterpret_cast<const uint4*>(res + vox * COUT);
#pragma unroll
          for (int q = 0; q < COUT / 8; ++q) {
            const uint4 rv = rp[q];
            const uint32_t rw[4] = {rv.x, rv.y, rv.z, rv.w};
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              const __nv_bfloat162 r2 = *reinterpret_cast<const __nv_bfloat162*>(&rw[e]);
              o[8 * q + 2 * e] += __low2float(r2);
              o[8 * q + 2 * e + 1] += __high2float(r2);
            }
          }
        }
        if constexpr (sizeof(OutT) == 4) {
          float4* op = reinterpret_cast<float4*>(out + vox * COUT);
#pragma unroll
          for (int q = 0; q < COUT / 4; ++q) op[q] = make_float4(o[4 * q], o[4 * q + 1], o[4 * q + 2], o[4 * q + 3]);
        } else {
          uint4* op = reinterpret_cast<uint4*>(out + vox * COUT);
#pragma unroll
          for (int q = 0; q < COUT / 8; ++q) {
            uint32_t pk[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              const __nv_bfloat162 b2 = __floats2bfloat162_rn(o[8 * q + 2 * e], o[8 * q + 2 * e + 1]);
              pk[e] = *reinterpret_cast<const uint32_t*>(&b2);
            }
            op[q] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
      __syncwarp();
      if (lane == 0) tc_arrive(acc_empty + acc);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  if (threadIdx.x == 0 && *abort) atomicExch(err, 1);
  if (warp == TC_MMA_WARP) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 128;\n" ::"r"(tmem));
}

// ---- weight gradient on tcgen05 -------------------------------------------------
//
// dW[tap][co][ci] = sum_v dout[v][co] in[v + off(tap)][ci] with the reduction (K) over 16 consecutive z voxels
// per MMA.  One operand, S, has 32 channels and is read at shifted voxels; the other, U (Cu = 16 or 32
// channels), at the tile's own voxels and at the levels above and below.  For the 32 -> Cout layers S is the
// input and U the output gradient; for the 16 -> 32 layer S is the output gradient and U the input, and the
// taps come out mirrored (sum_v dout[v] in[v + t] = sum_u dout[u - t] in[u]).
//
// Both operands are MN-major: a core matrix is 8 consecutive z voxels (K) x 8 channels (16 bytes), which is
// how channels-last volumes arrive, so cp.async copies 16-byte chunks straight into place.
//   A (M = 128): rows (l, c) = channel c of S on x line x + l - 1, l = 0..3 (l = 3 is a spare line whose
//     rows are discarded), at z + dz - 1.  S halo rows [level][line][chunk][z - 1 .. z + 16] with the line
//     pitch = 4 chunk planes, so the 16 core matrices of rows (l, chunk) sit one plane pitch apart; the z tap
//     dz is the descriptor's start address moved dz rows.
//   B (N = 3 Cu): columns (e, c) = channel c of U at level y + e - 1, e = 0..2, the levels a level pitch
//     apart in U's rows [column][level][chunk][z].
// One MMA per (level of the tile, x column, dz) accumulates D[dz] (128 x 3Cu fp32 in TMEM) over every tile
// of the persistent CTA; tap (dy, dz, dx) of D[dz][(l, c)][(e, c')] is (1 - e, dz - 1, l - 1) relative to U.
// Roles as in the forward kernel: warps 0-3 copy a tile's halo into a ring of stage buffers (register-staged
// 16-byte loads and stores) and arrive on `full`; warp 8 (one thread) issues the tile's MMAs and commits them to `empty`; warps 4-7 sum the tile's
// output gradient (the bias gradient) from the same buffer and arrive on `empty` too, and at the end read
// D from TMEM and add it to dw.  Every wait is bounded as in the forward kernel.
constexpr int WT_TXW = 8;               // x columns per tile
constexpr int WT_TY = 2;                // y levels per tile
constexpr int WT_TZ = 16;               // z voxels per tile = the K of one MMA
constexpr int WT_L = WT_TXW + 3;        // S halo lines x0 - 1 .. x0 + 9
constexpr int WT_ZR = WT_TZ + 2;        // S halo z rows
constexpr int WT_ZP = 19;               // S z pitch in 16-byte rows (odd: a warp's copies spread over all banks)
constexpr int WT_ZPU = 17;              // U z pitch
constexpr int WT_THREADS = 288;

template <int CU>
struct WtGeom {
  static constexpr int KCS = 4, KCU = CU / 8, UL = WT_TY + 2;
  static constexpr int SROWS = WT_TY * WT_L * KCS * WT_ZP;  // S halo rows of a stage
  static constexpr int XIP = UL * KCU * WT_ZPU + 1;         // U rows per x column (odd)
  static constexpr int BUF = SROWS + WT_TXW * XIP;          // 16-byte rows per stage
  static constexpr int NBUF = CU == 32 ? 3 : 4;
  static constexpr int NCOL = 3 * CU;                       // N of one MMA
  static constexpr int TCOLS = 3 * NCOL <= 256 ? 256 : 512; // TMEM columns (a power of two >= 3 NCOL)
  static constexpr size_t smem = (size_t)NBUF * BUF * 16 + (2 * NBUF + 1) * 8 + 16;
};

template <int CU, bool SWAP>
__global__ void __launch_bounds__(WT_THREADS, 1)
    k_conv_wgrad_tc(const __nv_bfloat16* __restrict__ sop, const __nv_bfloat16* __restrict__ uop,
                    float* __restrict__ dw, float* __restrict__ db, Vol v, int* __restrict__ err) {
  using G = WtGeom<CU>;
  constexpr int KCS = G::KCS, KCU = G::KCU, NBUF = G::NBUF, BUF = G::BUF, NCOL = G::NCOL;
  constexpr int CIN = SWAP ? CU : 32, COUT = SWAP ? 32 : CU;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint4* ring = reinterpret_cast<uint4*>(smem_raw);  // [NBUF][BUF]
  uint64_t* full = reinterpret_cast<uint64_t*>(ring + (size_t)NBUF * BUF);
  uint64_t* empty = full + NBUF;
  uint64_t* done = empty + NBUF;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(done + 1);
  volatile int* abort = reinterpret_cast<volatile int*>(tslot + 1);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

  if (threadIdx.x == 0) {
    for (int b = 0; b < NBUF; ++b) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(full + b)), "r"(TC_PRODUCERS));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 5;\n" ::"r"(smem_u32(empty + b)));  // MMAs + 4 warps
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(done)));
    *abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == TC_MMA_WARP) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tslot)),
                 "n"(G::TCOLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = *tslot;

  const int nty = (v.Y + WT_TY - 1) / WT_TY, ntz = v.Z / WT_TZ, ntx = v.X / WT_TXW;
  const int ntiles = nty * ntz * ntx;
  const int my_tiles = blockIdx.x < ntiles ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  auto tile_origin = [&](int s, int& y0, int& z0, int& x0) {
    const int tile = blockIdx.x + s * gridDim.x;
    const int xt = tile % ntx, rest = tile / ntx;
    x0 = xt * WT_TXW;
    z0 = (rest % ntz) * WT_TZ;
    y0 = (rest / ntz) * WT_TY;
  };

  if (warp < 4) {
    // ---- producers: tile s into buffer s % NBUF.  16-byte loads into registers, then 16-byte shared stores
    // (a warp's 32 loads cover 512 contiguous bytes and its stores hit every bank group four times), S first,
    // then U; the buffer is handed over as soon as its stores are done.
    const int p = threadIdx.x;
    constexpr int SCH = WT_TY * WT_ZR * WT_L * KCS, UCH = G::UL * WT_TZ * WT_TXW * KCU;
    constexpr int SPT = (SCH + TC_PRODUCERS - 1) / TC_PRODUCERS, UPT = (UCH + TC_PRODUCERS - 1) / TC_PRODUCERS;
    for (int s = 0; s < my_tiles; ++s) {
      if (s >= NBUF && !tc_wait(empty + s % NBUF, (uint32_t)((s / NBUF - 1) & 1), abort)) break;
      int y0, z0, x0;
      tile_origin(s, y0, z0, x0);
      uint4* buf = ring + (size_t)(s % NBUF) * BUF;
      {  // S: rows ((t L + line) 4 + chunk) ZP + zr; levels y0 + t past the top are zeros
        uint4 r[SPT];
        int row[SPT];
#pragma unroll
        for (int i = 0; i < SPT; ++i) {
          const int c = p + i * TC_PRODUCERS;
          r[i] = make_uint4(0u, 0u, 0u, 0u);
          row[i] = -1;
          if (c < SCH) {
            const int kc = c % KCS, line = (c / KCS) % WT_L, r2 = c / (KCS * WT_L);
            const int zr = r2 % WT_ZR, t = r2 / WT_ZR;
            const int gy = y0 + t;
            int gz = z0 + zr - 1, gx = x0 + line - 1;
            gz = gz < 0 ? gz + v.Z : (gz >= v.Z ? gz - v.Z : gz);
            gx = gx < 0 ? gx + v.X : (gx >= v.X ? gx - v.X : gx);
            row[i] = ((t * WT_L + line) * KCS + kc) * WT_ZP + zr;
            if (gy < v.Y)
              r[i] = __ldg(reinterpret_cast<const uint4*>(sop + (((size_t)gy * v.Z + gz) * v.X + gx) * 32 + kc * 8));
          }
        }
#pragma unroll
        for (int i = 0; i < SPT; ++i)
          if (row[i] >= 0) buf[row[i]] = r[i];
      }
      {  // U: rows SROWS + column XIP + (level KCU + chunk) ZPU + z; levels y0 - 1 .. y0 + 2, zeros outside
        uint4 r[UPT];
        int row[UPT];
#pragma unroll
        for (int i = 0; i < UPT; ++i) {
          const int c = p + i * TC_PRODUCERS;
          r[i] = make_uint4(0u, 0u, 0u, 0u);
          row[i] = -1;
          if (c < UCH) {
            const int kcu = c % KCU, xi = (c / KCU) % WT_TXW, r2 = c / (KCU * WT_TXW);
            const int z = r2 % WT_TZ, lev = r2 / WT_TZ;
            const int gy = y0 + lev - 1;
            row[i] = G::SROWS + xi * G::XIP + (lev * KCU + kcu) * WT_ZPU + z;
            if (gy >= 0 && gy < v.Y)
              r[i] = __ldg(reinterpret_cast<const uint4*>(uop + (((size_t)gy * v.Z + z0 + z) * v.X + x0 + xi) * CU +
                                                          kcu * 8));
          }
        }
#pragma unroll
        for (int i = 0; i < UPT; ++i)
          if (row[i] >= 0) buf[row[i]] = r[i];
      }
      asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
      tc_arrive(full + s % NBUF);
    }
  } else if (warp == TC_MMA_WARP) {
    // ---- MMA issue: one thread
    if (lane == 0) {
      // kind::f16 (bf16 operands, fp32 D), M = 128, N = 3 Cu, A and B MN-major (bits 15, 16)
      const uint32_t idesc = tc_idesc(128, NCOL) | (1u << 15) | (1u << 16);
      const uint64_t a0 = tc_smem_desc(smem_u32(ring), 128, WT_ZP * 16);
      const uint64_t b0 = tc_smem_desc(smem_u32(ring + G::SROWS), 128, WT_ZPU * 16);
      for (int s = 0; s < my_tiles; ++s) {
        if (!tc_wait(full + s % NBUF, (uint32_t)((s / NBUF) & 1), abort)) break;
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        const uint64_t boff = (uint64_t)((s % NBUF) * BUF);  // start address in 16-byte units
#pragma unroll 1
        for (int t = 0; t < WT_TY; ++t) {
#pragma unroll
          for (int xi = 0; xi < WT_TXW; ++xi) {
            const uint64_t bd = b0 + boff + (uint64_t)(xi * G::XIP + t * KCU * WT_ZPU);
            const uint32_t accum = (s > 0 || t > 0 || xi > 0) ? 1u : 0u;
#pragma unroll
            for (int dz = 0; dz < 3; ++dz) {
              const uint64_t ad = a0 + boff + (uint64_t)((t * WT_L + xi) * KCS * WT_ZP + dz);
              asm volatile(
                  "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                  "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem + (uint32_t)(dz * NCOL)),
                  "l"(ad), "l"(bd), "r"(idesc), "r"(accum));
            }
          }
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
            smem_u32(empty + s % NBUF)));
      }
      // `done` completes once every MMA issued above has
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
          smem_u32(done)));
      volatile int no_abort = 0;
      tc_wait(done, 0u, &no_abort);
      if (no_abort) *abort = 1;
    }
    __syncwarp();
  } else {
    // ---- warps 4-7: bias gradient from each stage, then D -> dw
    const int g = warp & 3, e = threadIdx.x - 128;
    constexpr int KB = SWAP ? KCS : KCU;  // 16-byte chunks per output-gradient voxel
    const int kb = e % KB;                // this thread's chunk (128 is a multiple of KB)
    float bacc[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) bacc[i] = 0.f;
    for (int s = 0; s < my_tiles; ++s) {
      if (!tc_wait(full + s % NBUF, (uint32_t)((s / NBUF) & 1), abort)) break;
      const uint4* buf = ring + (size_t)(s % NBUF) * BUF;
      for (int c = e; c < WT_TY * WT_TXW * WT_TZ * KB; c += 128) {
        const int xi = (c / KB) % WT_TXW, r2 = c / (KB * WT_TXW);
        const int z = r2 % WT_TZ, t = r2 / WT_TZ;
        const size_t row = SWAP ? ((size_t)(t * WT_L + xi + 1) * KCS + kb) * WT_ZP + z + 1
                                : G::SROWS + (size_t)xi * G::XIP + ((t + 1) * KCU + kb) * WT_ZPU + z;
        const uint4 q = buf[row];
        const uint32_t w4[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const __nv_bfloat162 b2 = *reinterpret_cast<const __nv_bfloat162*>(&w4[i]);
          bacc[2 * i] += __low2float(b2);
          bacc[2 * i + 1] += __high2float(b2);
        }
      }
      __syncwarp();
      if (lane == 0) tc_arrive(empty + s % NBUF);
    }
#pragma unroll
    for (int off = KB; off < 32; off <<= 1)
#pragma unroll
      for (int i = 0; i < 8; ++i) bacc[i] += __shfl_xor_sync(0xffffffffu, bacc[i], off);
    if (lane < KB) {
#pragma unroll
      for (int i = 0; i < 8; ++i) atomicAdd(db + kb * 8 + i, bacc[i]);
    }
    // D -> dw: warp 4 + g reads TMEM lanes 32 g .. 32 g + 31 = rows (l = g, channel = lane) of S
    const bool ok = tc_wait(done, 0u, abort);
    const bool go = __all_sync(0xffffffffu, ok && !*abort) && g < 3 && my_tiles > 0;
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (go) {
#pragma unroll 1
      for (int dz = 0; dz < 3; ++dz) {
#pragma unroll 1
        for (int c16 = 0; c16 < NCOL / 16; ++c16) {
          uint32_t r[16];
          const uint32_t taddr = tmem + ((uint32_t)(g * 32) << 16) + (uint32_t)(dz * NCOL + c16 * 16);
          asm volatile(
              "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
              "[%16];\n"
              : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                "=r"(r[15])
              : "r"(taddr));
          asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int n = c16 * 16 + j, lev = n / CU, uc = n % CU;
            // tap (dy, dz, dx) of S relative to U is (1 - lev, dz - 1, g - 1); mirrored when S is dout
            const int tap = SWAP ? lev * 9 + (2 - dz) * 3 + (2 - g) : (2 - lev) * 9 + dz * 3 + g;
            const int co = SWAP ? lane : uc, ci = SWAP ? uc : lane;
            atomicAdd(dw + ((size_t)tap * COUT + co) * CIN + ci, __uint_as_float(r[j]));
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  if (threadIdx.x == 0 && *abort) atomicExch(err, 1);
  if (warp == TC_MMA_WARP)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "n"(G::TCOLS));
}

// ---- launchers ---------------------------------------------------------------

int num_sms() {
  int dev = 0, n = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  return n > 0 ? n : 1;
}

__device__ int g_tc_err;  // set when a tcgen05 convolution's mbarrier wait ran out

template <int CIN, int COUT>
constexpr size_t tc_smem() {
  // halo ring, weights, 2 TC_NBUF + 4 mbarriers, the TMEM address and the abort flag
  return (size_t)TC_NBUF * (CIN / 8) * TC_KP * 16 + (size_t)27 * (CIN / 8) * COUT * 16 + (2 * TC_NBUF + 4) * 8 + 16;
}

template <int CIN, int COUT, typename OutT>
cudaError_t conv_fwd_tc(const void* in, const void* w, const float* bias, void* out, const void* res,
                        const void* gate, int epi, Vol v, cudaStream_t st) {
  auto k = k_conv_fwd_tc<CIN, COUT, OutT>;
  const size_t sm = tc_smem<CIN, COUT>();
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  int* err = nullptr;
  e = cudaGetSymbolAddress((void**)&err, g_tc_err);
  if (e != cudaSuccess) return e;
  const int ntiles = v.Y * (v.Z / TC_TZ) * (v.X / TX);
  const int grid = ntiles < num_sms() ? ntiles : num_sms();
  k<<<grid, TC_THREADS, sm, st>>>((const __nv_bfloat16*)in, (const __nv_bfloat16*)w, bias, (OutT*)out,
                           (const __nv_bfloat16*)res, (const __nv_bfloat16*)gate, epi, v, err);
  return cudaGetLastError();
}

template <int CIN, int COUT>
constexpr size_t fwd_smem() {
  return (size_t)(27 * COUT * (CIN + 8) + HROWS * (CIN + 8)) * 2;
}
template <int CIN, int COUT>
constexpr size_t wgrad_smem() {
  return (size_t)(HROWS * (CIN + 8) + TZ * TX * (COUT + 8)) * 2 + COUT * 4;
}

template <int CIN, int COUT, typename OutT>
cudaError_t conv_fwd(const void* in, const void* w, const float* bias, void* out, const void* res, const void* gate,
                     int epi, Vol v, cudaStream_t st) {
  auto k = k_conv_fwd<CIN, COUT, OutT>;
  const size_t sm = fwd_smem<CIN, COUT>();
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  const int ntiles = v.Y * (v.Z / TZ) * (v.X / TX);
  const int grid = ntiles < num_sms() ? ntiles : num_sms();
  k<<<grid, TZ * 32, sm, st>>>((const __nv_bfloat16*)in, (const __nv_bfloat16*)w, bias, (OutT*)out,
                               (const __nv_bfloat16*)res, (const __nv_bfloat16*)gate, epi, v);
  return cudaGetLastError();
}

template <int CIN, int COUT>
cudaError_t conv_wgrad(const void* in, const void* dout, float* dw, float* db, Vol v, cudaStream_t st) {
  auto k = k_conv_wgrad<CIN, COUT>;
  const size_t sm = wgrad_smem<CIN, COUT>();
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  const int ntiles = v.Y * (v.Z / TZ) * (v.X / TX);
  const int grid = ntiles < num_sms() ? ntiles : num_sms();
  k<<<grid, WG_WARPS * 32, sm, st>>>((const __nv_bfloat16*)in, (const __nv_bfloat16*)dout, dw, db, v);
  return cudaGetLastError();
}

template <int CU, bool SWAP>
cudaError_t conv_wgrad_tc(const void* sop, const void* uop, float* dw, float* db, Vol v, cudaStream_t st) {
  auto k = k_conv_wgrad_tc<CU, SWAP>;
  const size_t sm = WtGeom<CU>::smem;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  int* err = nullptr;
  e = cudaGetSymbolAddress((void**)&err, g_tc_err);
  if (e != cudaSuccess) return e;
  const int ntiles = ((v.Y + WT_TY - 1) / WT_TY) * (v.Z / WT_TZ) * (v.X / WT_TXW);
  const int grid = ntiles < num_sms() ? ntiles : num_sms();
  k<<<grid, WT_THREADS, sm, st>>>((const __nv_bfloat16*)sop, (const __nv_bfloat16*)uop, dw, db, v, err);
  return cudaGetLastError();
}

}  // namespace sr
}  // namespace lh

// ---- C ABI (include/lh_srnet.h) ------------------------------------------------

using lh::sr::Vol;

namespace {
int sr_check_vol(int X, int Y, int Z) {
  if (X <= 0 || Y <= 0 || Z <= 0 || X % lh::sr::TX || Z % lh::sr::TZ) {
    lh::set_init_error("lh_sr: volume needs X a multiple of 32 and Z a multiple of 8");
    return LH_EINVAL;
  }
  return LH_OK;
}
int sr_cuda(cudaError_t e) {
  if (e == cudaSuccess) return LH_OK;
  lh::set_init_error(cudaGetErrorString(e));
  return LH_ECUDA;
}
bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }
}  // namespace

extern "C" {

int lh_sr_conv_fwd(int32_t cin, int32_t cout, const void* in, const void* w, const float* bias, void* out,
                   int32_t out_f32, const void* res, const void* gate, int32_t flags, int32_t X, int32_t Y, int32_t Z,
                   void* stream) {
  int rc = sr_check_vol(X, Y, Z);
  if (rc) return rc;
  if (!in || !w || !out || !aligned16(in) || !aligned16(w) || ((flags & 2) && !res) || ((flags & 4) && !gate) ||
      ((flags & 8) && !bias)) {
    lh::set_init_error("lh_sr_conv_fwd: missing or misaligned pointer");
    return LH_EINVAL;
  }
  const Vol v{X, Y, Z};
  cudaStream_t st = (cudaStream_t)stream;
  using bf = __nv_bfloat16;
  if (cin == 16 && cout == 32 && !out_f32) return sr_cuda(lh::sr::conv_fwd<16, 32, bf>(in, w, bias, out, res, gate, flags, v, st));
  if (cin == 32 && cout == 32 && !out_f32) return sr_cuda(lh::sr::conv_fwd<32, 32, bf>(in, w, bias, out, res, gate, flags, v, st));
  if (cin == 32 && cout == 16 && !out_f32) return sr_cuda(lh::sr::conv_fwd<32, 16, bf>(in, w, bias, out, res, gate, flags, v, st));
  if (cin == 32 && cout == 16 && out_f32) return sr_cuda(lh::sr::conv_fwd<32, 16, float>(in, w, bias, out, res, gate, flags, v, st));
  lh::set_init_error("lh_sr_conv_fwd: channel pair not built (16->32, 32->32, 32->16)");
  return LH_EINVAL;
}

int lh_sr_conv_fwd_tc(int32_t cin, int32_t cout, const void* in, const void* w, const float* bias, void* out,
                      int32_t out_f32, const void* res, const void* gate, int32_t flags, int32_t X, int32_t Y,
                      int32_t Z, void* stream) {
  int rc = sr_check_vol(X, Y, Z);
  if (rc) return rc;
  if (Z % lh::sr::TC_TZ) {
    lh::set_init_error("lh_sr_conv_fwd_tc: Z must be a multiple of 8");
    return LH_EINVAL;
  }
  if (!in || !w || !out || !aligned16(in) || !aligned16(w) || !aligned16(out) || ((flags & 2) && !aligned16(res)) ||
      ((flags & 4) && !aligned16(gate)) || ((flags & 8) && !bias)) {
    lh::set_init_error("lh_sr_conv_fwd_tc: missing or misaligned pointer");
    return LH_EINVAL;
  }
  const Vol v{X, Y, Z};
  cudaStream_t st = (cudaStream_t)stream;
  using bf = __nv_bfloat16;
  if (cin == 16 && cout == 32 && !out_f32) return sr_cuda(lh::sr::conv_fwd_tc<16, 32, bf>(in, w, bias, out, res, gate, flags, v, st));
  if (cin == 32 && cout == 32 && !out_f32) return sr_cuda(lh::sr::conv_fwd_tc<32, 32, bf>(in, w, bias, out, res, gate, flags, v, st));
  if (cin == 32 && cout == 16 && !out_f32) return sr_cuda(lh::sr::conv_fwd_tc<32, 16, bf>(in, w, bias, out, res, gate, flags, v, st));
  if (cin == 32 && cout == 16 && out_f32) return sr_cuda(lh::sr::conv_fwd_tc<32, 16, float>(in, w, bias, out, res, gate, flags, v, st));
  lh::set_init_error("lh_sr_conv_fwd_tc: channel pair not built (16->32, 32->32, 32->16)");
  return LH_EINVAL;
}

int lh_sr_tc_status(int32_t* timed_out) {
  if (!timed_out) return LH_EINVAL;
  int v = 0;
  cudaError_t e = cudaMemcpyFromSymbol(&v, lh::sr::g_tc_err, sizeof v);
  if (e != cudaSuccess) return sr_cuda(e);
  *timed_out = v;
  const int zero = 0;
  return sr_cuda(cudaMemcpyToSymbol(lh::sr::g_tc_err, &zero, sizeof zero));
}

int lh_sr_conv_wgrad(int32_t cin, int32_t cout, const void* in, const void* dout, float* dw, float* db, int32_t X,
                     int32_t Y, int32_t Z, void* stream) {
  int rc = sr_check_vol(X, Y, Z);
  if (rc) return rc;
  if (!in || !dout || !dw || !db || !aligned16(in) || !aligned16(dout)) {
    lh::set_init_error("lh_sr_conv_wgrad: missing or misaligned pointer");
    return LH_EINVAL;
  }
  const Vol v{X, Y, Z};
  cudaStream_t st = (cudaStream_t)stream;
  if (cin == 16 && cout == 32) return sr_cuda(lh::sr::conv_wgrad<16, 32>(in, dout, dw, db, v, st));
  if (cin == 32 && cout == 32) return sr_cuda(lh::sr::conv_wgrad<32, 32>(in, dout, dw, db, v, st));
  if (cin == 32 && cout == 16) return sr_cuda(lh::sr::conv_wgrad<32, 16>(in, dout, dw, db, v, st));
  lh::set_init_error("lh_sr_conv_wgrad: channel pair not built (16->32, 32->32, 32->16)");
  return LH_EINVAL;
}

int lh_sr_conv_wgrad_tc(int32_t cin, int32_t cout, const void* in, const void* dout, float* dw, float* db,
                        int32_t X, int32_t Y, int32_t Z, void* stream) {
  int rc = sr_check_vol(X, Y, Z);
  if (rc) return rc;
  if (Z % lh::sr::WT_TZ) {
    lh::set_init_error("lh_sr_conv_wgrad_tc: Z must be a multiple of 16");
    return LH_EINVAL;
  }
  if (!in || !dout || !dw || !db || !aligned16(in) || !aligned16(dout)) {
    lh::set_init_error("lh_sr_conv_wgrad_tc: missing or misaligned pointer");
    return LH_EINVAL;
  }
  const Vol v{X, Y, Z};
  cudaStream_t st = (cudaStream_t)stream;
  // the 32-channel operand is the shifted one: the input for 32 -> Cout, the output gradient for 16 -> 32
  if (cin == 32 && cout == 32) return sr_cuda(lh::sr::conv_wgrad_tc<32, false>(in, dout, dw, db, v, st));
  if (cin == 32 && cout == 16) return sr_cuda(lh::sr::conv_wgrad_tc<16, false>(in, dout, dw, db, v, st));
  if (cin == 16 && cout == 32) return sr_cuda(lh::sr::conv_wgrad_tc<16, true>(dout, in, dw, db, v, st));
  lh::set_init_error("lh_sr_conv_wgrad_tc: channel pair not built (16->32, 32->32, 32->16)");
  return LH_EINVAL;
}

int lh_sr_flip_weights(int32_t cin, int32_t cout, const void* w, void* wt, void* stream) {
  if (!w || !wt || cin <= 0 || cout <= 0) return LH_EINVAL;
  const int n = 27 * cin * cout;
  lh::sr::k_flip_weights<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16*)w,
                                                                          (__nv_bfloat16*)wt, cin, cout);
  return sr_cuda(cudaGetLastError());
}

int lh_sr_mse(const float* corr, const float* base, const float* target, void* dcorr, double* loss, int64_t nvox,
              void* stream) {
  if (!corr || !base || !target || !dcorr || !loss || nvox <= 0 || !aligned16(dcorr)) return LH_EINVAL;
  const int blocks = (int)((nvox + 255) / 256 < 4 * 1024 ? (nvox + 255) / 256 : 4 * 1024);
  lh::sr::k_mse<<<blocks, 256, 0, (cudaStream_t)stream>>>(corr, base, target, (__nv_bfloat16*)dcorr, loss, nvox,
                                                          1.0f / (3.0f * (float)nvox));
  return sr_cuda(cudaGetLastError());
}

int lh_sr_adam(float* p, const float* g, float* m, float* v, void* p_bf16, int32_t n, float lr, float beta1,
               float beta2, float eps, float weight_decay, int32_t step, void* stream) {
  if (!p || !g || !m || !v || n <= 0 || step < 1) return LH_EINVAL;
  const float bc1 = 1.f - powf(beta1, (float)step), bc2 = 1.f - powf(beta2, (float)step);
  const int blocks = (n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024;
  lh::sr::k_adam<<<blocks, 256, 0, (cudaStream_t)stream>>>(p, g, m, v, (__nv_bfloat16*)p_bf16, n, lr, beta1, beta2,
                                                           eps, weight_decay, bc1, bc2);
  return sr_cuda(cudaGetLastError());
}

}  // extern "C"
