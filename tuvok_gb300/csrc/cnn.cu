// cnn.cu -- kernels of the learned reconstruction network: 3x3 convolutions on
// the tensor cores (BF16 operands, FP32 accumulation) forward, backward-data
// and backward-weights, 2x2 average pooling, 2x nearest upsampling, the
// pixel-shuffle head that adds the network's residual to the bilinear upscale
// of the reduced frame, the loss and Adam.
//
// Layout: activations NHWC (channels innermost), BF16; weights of a layer as
// [tap = ky * 3 + kx][cout][cin] (cin innermost), FP32 masters and BF16 copies.
// A convolution is an implicit GEMM: M = output pixels, N = output channels,
// K = 9 taps x input channels.  Channel counts that are multiples of 16 run on
// tcgen05 (conv3x3_tc_kernel: 16x8-pixel patches as M = 128, accumulators in
// tensor memory); the others on mma.sync.m16n8k16, one CTA (4 warps) per 8x8
// patch or (8 warps) per 16x16 patch, the halo and the weights staged in shared
// memory.  The skip connections of the U-Net concatenate two tensors along
// channels; the convolution reads them in place (x1: c1 channels, x2: c2).
#include <cuda_bf16.h>

#include <algorithm>
#include <cstdint>
#include <mutex>

#include "tvk_internal.h"

namespace tvk {
namespace {

constexpr int kThreads = 128;

__device__ __forceinline__ uint32_t pack_bf16(__nv_bfloat16 lo, __nv_bfloat16 hi) {
  return uint32_t(__bfloat16_as_ushort(lo)) | (uint32_t(__bfloat16_as_ushort(hi)) << 16);
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0,
                                         uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// ------------------------------------------------------------- convolution

// Output of a convolution: BF16 (with bias and LeakyReLU) or FP32 (optionally
// added to what is there, for gradients that sum over several consumers), and
// optionally split by channel into two tensors (gradients of a concatenation).
struct ConvArgs {
  const __nv_bfloat16* x1;
  const __nv_bfloat16* x2;
  int c1, c2;                 // input channels of x1, x2 (c2 may be 0)
  int n, h, w;                // batch and spatial size (same in and out)
  const __nv_bfloat16* wt;    // [9][cout][c1 + c2]
  const float* bias;          // [cout] or null
  int cout;
  float slope;                // LeakyReLU negative slope; < 0: no activation
  __nv_bfloat16* y_bf16;      // BF16 output [n][h][w][cout] or null
  float* y_f32;               // FP32 output (first split) or null
  float* y2_f32;              // FP32 output of channels >= split or null
  int split;                  // channel where y2 starts (== cout: no split)
  int accumulate;             // FP32 outputs: add to the existing values
  int up1, h1, w1;            // x1 read through a clamped 2x nearest upsampling of h1 x w1
  // tcgen05 kernel only: the 16 output channels are a pixel-shuffled RGBA
  // residual (channel c * 4 + dy * 2 + dx of pixel (y, x) -> channel c of pixel
  // (2y + dy, 2x + dx)) added in place to this FP32 [oh][ow][4] image
  float* shuffle;
  int oh, ow;
};

// Pixel index of x1 for output-grid pixel (yy, xx) of image img.
__device__ __forceinline__ size_t x1_pixel(const ConvArgs& a, int img, int yy, int xx) {
  if (!a.up1) return (size_t(img) * a.h + yy) * a.w + xx;
  return (size_t(img) * a.h1 + min(yy >> 1, a.h1 - 1)) * a.w1 + min(xx >> 1, a.w1 - 1);
}

template <int kNT>  // n-tiles of 8 output channels
__global__ void __launch_bounds__(kThreads) conv3x3_kernel(const ConvArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int cin = a.c1 + a.c2;
  const int cpad = cin + 8;  // row pitch of the halo (breaks bank conflicts)
  __nv_bfloat16* halo = reinterpret_cast<__nv_bfloat16*>(smem_raw);       // [100][cpad]
  __nv_bfloat16* wsm = halo + 100 * cpad;                                // [cout][cpad]
  const int tiles_x = (a.w + 7) / 8, tiles_y = (a.h + 7) / 8;
  const int t = blockIdx.x;
  const int img = t / (tiles_x * tiles_y);
  const int ty = (t / tiles_x) % tiles_y, tx = t % tiles_x;
  const int y0 = ty * 8 - 1, x0 = tx * 8 - 1;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int g = lane >> 2, q = lane & 3;

  // 10x10 halo of the input, zero outside the image; two channels per thread step
  const int halo_words = 100 * (cin / 2);
  for (int i = tid; i < halo_words; i += kThreads) {
    const int pix = i / (cin / 2), c = (i % (cin / 2)) * 2;
    const int yy = y0 + pix / 10, xx = x0 + pix % 10;
    uint32_t v = 0;
    if (yy >= 0 && yy < a.h && xx >= 0 && xx < a.w) {
      const size_t p = (size_t(img) * a.h + yy) * a.w + xx;
      v = c < a.c1 ? *reinterpret_cast<const uint32_t*>(a.x1 + x1_pixel(a, img, yy, xx) * a.c1 + c)
                   : *reinterpret_cast<const uint32_t*>(a.x2 + p * a.c2 + (c - a.c1));
    }
    *reinterpret_cast<uint32_t*>(halo + pix * cpad + c) = v;
  }

  float acc[kNT][4];
#pragma unroll
  for (int j = 0; j < kNT; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
  // this thread's two pixel rows of the warp's 16 pixels (patch rows 2w, 2w+1)
  const int pr0 = 2 * warp, pr1 = 2 * warp + 1, pc = g;
  const int cout_pad = kNT * 8;
  for (int tap = 0; tap < 9; ++tap) {
    __syncthreads();  // halo written / previous tap's weights no longer read
    const __nv_bfloat16* wtap = a.wt + size_t(tap) * a.cout * cin;
    for (int i = tid; i < cout_pad * (cin / 2); i += kThreads) {
      const int co = i / (cin / 2), c = (i % (cin / 2)) * 2;
      const uint32_t v = co < a.cout ? *reinterpret_cast<const uint32_t*>(wtap + co * cin + c) : 0u;
      *reinterpret_cast<uint32_t*>(wsm + co * cpad + c) = v;
    }
    __syncthreads();
    const int ky = tap / 3, kx = tap % 3;
    const __nv_bfloat16* r0 = halo + ((pr0 + ky) * 10 + pc + kx) * cpad;
    const __nv_bfloat16* r1 = halo + ((pr1 + ky) * 10 + pc + kx) * cpad;
    for (int k0 = 0; k0 < cin; k0 += 16) {
      uint32_t af[4];
      af[0] = *reinterpret_cast<const uint32_t*>(r0 + k0 + 2 * q);
      af[1] = *reinterpret_cast<const uint32_t*>(r1 + k0 + 2 * q);
      af[2] = *reinterpret_cast<const uint32_t*>(r0 + k0 + 8 + 2 * q);
      af[3] = *reinterpret_cast<const uint32_t*>(r1 + k0 + 8 + 2 * q);
#pragma unroll
      for (int j = 0; j < kNT; ++j) {
        const __nv_bfloat16* wr = wsm + (j * 8 + g) * cpad + k0 + 2 * q;
        mma_bf16(acc[j], af, *reinterpret_cast<const uint32_t*>(wr),
                 *reinterpret_cast<const uint32_t*>(wr + 8));
      }
    }
  }

  // epilogue: rows g (pixel row pr0) and g + 8 (pixel row pr1), columns 2q, 2q+1
  const int oy0 = ty * 8 + pr0, oy1 = ty * 8 + pr1, ox = tx * 8 + pc;
#pragma unroll
  for (int j = 0; j < kNT; ++j) {
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const int oy = half ? oy1 : oy0;
      if (oy >= a.h || ox >= a.w) continue;
      const size_t p = (size_t(img) * a.h + oy) * a.w + ox;
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const int co = j * 8 + 2 * q + e;
        if (co >= a.cout) continue;
        float v = acc[j][half * 2 + e];
        if (a.bias) v += a.bias[co];
        if (a.slope >= 0.0f && v < 0.0f) v *= a.slope;
        if (a.y_bf16) a.y_bf16[p * a.cout + co] = __float2bfloat16_rn(v);
        if (co < a.split) {
          if (a.y_f32) {
            float* o = a.y_f32 + p * a.split + co;
            *o = a.accumulate ? *o + v : v;
          }
        } else if (a.y2_f32) {
          const int c2n = a.cout - a.split;
          float* o = a.y2_f32 + p * c2n + (co - a.split);
          *o = a.accumulate ? *o + v : v;
        }
      }
    }
  }
}

// The same convolution for large images: a CTA of 8 warps computes a 16x16
// pixel patch (each warp two pixel rows of 16 = two m16 tiles that share every
// B fragment), and with kAllTaps the weights of all 9 taps are staged once, so
// the tap loop runs without barriers.
constexpr int kWideThreads = 256;
constexpr int kWideTile = 16, kWideHalo = kWideTile + 2;

template <int kNT, bool kAllTaps>
__global__ void __launch_bounds__(kWideThreads) conv3x3_wide_kernel(const ConvArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int cin = a.c1 + a.c2;
  const int cpad = cin + 8;
  const int cw = cin / 2;  // 32-bit words per pixel
  __nv_bfloat16* halo = reinterpret_cast<__nv_bfloat16*>(smem_raw);   // [18 * 18][cpad]
  __nv_bfloat16* wsm = halo + kWideHalo * kWideHalo * cpad;           // [taps][cout_pad][cpad]
  const int tiles_x = (a.w + kWideTile - 1) / kWideTile;
  const int tiles_y = (a.h + kWideTile - 1) / kWideTile;
  const int t = blockIdx.x;
  const int img = t / (tiles_x * tiles_y);
  const int ty = (t / tiles_x) % tiles_y, tx = t % tiles_x;
  const int y0 = ty * kWideTile - 1, x0 = tx * kWideTile - 1;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int g = lane >> 2, q = lane & 3;
  constexpr int cout_pad = kNT * 8;

  for (int i = tid; i < kWideHalo * kWideHalo * cw; i += kWideThreads) {
    const int pix = i / cw, c = (i % cw) * 2;
    const int yy = y0 + pix / kWideHalo, xx = x0 + pix % kWideHalo;
    uint32_t v = 0;
    if (yy >= 0 && yy < a.h && xx >= 0 && xx < a.w) {
      const size_t p = (size_t(img) * a.h + yy) * a.w + xx;
      v = c < a.c1 ? *reinterpret_cast<const uint32_t*>(a.x1 + x1_pixel(a, img, yy, xx) * a.c1 + c)
                   : *reinterpret_cast<const uint32_t*>(a.x2 + p * a.c2 + (c - a.c1));
    }
    *reinterpret_cast<uint32_t*>(halo + pix * cpad + c) = v;
  }
  auto load_tap = [&](int tap, __nv_bfloat16* dst) {
    const __nv_bfloat16* wtap = a.wt + size_t(tap) * a.cout * cin;
    for (int i = tid; i < cout_pad * cw; i += kWideThreads) {
      const int co = i / cw, c = (i % cw) * 2;
      const uint32_t v = co < a.cout ? *reinterpret_cast<const uint32_t*>(wtap + co * cin + c) : 0u;
      *reinterpret_cast<uint32_t*>(dst + co * cpad + c) = v;
    }
  };
  if (kAllTaps) {
    for (int tap = 0; tap < 9; ++tap) load_tap(tap, wsm + tap * cout_pad * cpad);
    __syncthreads();
  }

  float acc[2][kNT][4];
#pragma unroll
  for (int m = 0; m < 2; ++m)
#pragma unroll
    for (int j = 0; j < kNT; ++j) acc[m][j][0] = acc[m][j][1] = acc[m][j][2] = acc[m][j][3] = 0.0f;
  const int pr0 = 2 * warp, pr1 = 2 * warp + 1;
  for (int tap = 0; tap < 9; ++tap) {
    const __nv_bfloat16* wt_s = wsm;
    if (kAllTaps) {
      wt_s = wsm + tap * cout_pad * cpad;
    } else {
      __syncthreads();  // halo written / previous tap's weights no longer read
      load_tap(tap, wsm);
      __syncthreads();
    }
    const int ky = tap / 3, kx = tap % 3;
    for (int k0 = 0; k0 < cin; k0 += 16) {
      uint32_t af[2][4];
#pragma unroll
      for (int m = 0; m < 2; ++m) {
        const __nv_bfloat16* r0 = halo + ((pr0 + ky) * kWideHalo + m * 8 + g + kx) * cpad;
        const __nv_bfloat16* r1 = halo + ((pr1 + ky) * kWideHalo + m * 8 + g + kx) * cpad;
        af[m][0] = *reinterpret_cast<const uint32_t*>(r0 + k0 + 2 * q);
        af[m][1] = *reinterpret_cast<const uint32_t*>(r1 + k0 + 2 * q);
        af[m][2] = *reinterpret_cast<const uint32_t*>(r0 + k0 + 8 + 2 * q);
        af[m][3] = *reinterpret_cast<const uint32_t*>(r1 + k0 + 8 + 2 * q);
      }
#pragma unroll
      for (int j = 0; j < kNT; ++j) {
        const __nv_bfloat16* wr = wt_s + (j * 8 + g) * cpad + k0 + 2 * q;
        const uint32_t b0 = *reinterpret_cast<const uint32_t*>(wr);
        const uint32_t b1 = *reinterpret_cast<const uint32_t*>(wr + 8);
        mma_bf16(acc[0][j], af[0], b0, b1);
        mma_bf16(acc[1][j], af[1], b0, b1);
      }
    }
  }

  // epilogue: m-tile m covers pixel columns 8m .. 8m+7; rows g (pr0), g + 8 (pr1)
#pragma unroll
  for (int m = 0; m < 2; ++m) {
    const int ox = tx * kWideTile + m * 8 + g;
#pragma unroll
    for (int j = 0; j < kNT; ++j) {
#pragma unroll
      for (int half = 0; half < 2; ++half) {
        const int oy = ty * kWideTile + (half ? pr1 : pr0);
        if (oy >= a.h || ox >= a.w) continue;
        const size_t p = (size_t(img) * a.h + oy) * a.w + ox;
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          const int co = j * 8 + 2 * q + e;
          if (co >= a.cout) continue;
          float v = acc[m][j][half * 2 + e];
          if (a.bias) v += a.bias[co];
          if (a.slope >= 0.0f && v < 0.0f) v *= a.slope;
          if (a.y_bf16) a.y_bf16[p * a.cout + co] = __float2bfloat16_rn(v);
          if (co < a.split) {
            if (a.y_f32) {
              float* o = a.y_f32 + p * a.split + co;
              *o = a.accumulate ? *o + v : v;
            }
          } else if (a.y2_f32) {
            const int c2n = a.cout - a.split;
            float* o = a.y2_f32 + p * c2n + (co - a.split);
            *o = a.accumulate ? *o + v : v;
          }
        }
      }
    }
  }
}

// ------------------------------------------------ convolution on tcgen05 / TMEM
//
// The same convolution on the fifth-generation tensor cores.  A CTA of 8 warps
// owns a 16 x 8 output patch = the M = 128 rows of one tcgen05.mma.kind::f16
// (BF16 operands, FP32 accumulator in tensor memory), N = all output channels,
// and loops over patches (persistent grid).  Shared memory holds, in the
// no-swizzle K-major core-matrix layout (8 rows x 16 bytes per core matrix):
//   halo    [cin / 8][18][10][8]  the patch's input with a 1-pixel border
//   weights [9][cin / 8][cout][8] all taps, loaded once per CTA
// so the A operand of tap (ky, kx) is the halo itself, offset by
// (ky * 10 + kx) * 16 bytes: 8-row groups (patch rows) 160 bytes apart, K core
// matrices (channel octets) 2880 bytes apart.  No im2col copy is made.  One
// thread issues the 9 x cin / 16 MMAs of a patch and commits them to an
// mbarrier; the warps then read their 32 TMEM lanes (pixels) and run the
// epilogue of the other kernels.  The halos of the following patches stream in
// with cp.async meanwhile, through a ring of up to 4 buffers.
constexpr int kTcRows = 16, kTcCols = 8;                  // output patch
constexpr int kTcHR = kTcRows + 2, kTcHC = kTcCols + 2;  // halo
constexpr uint32_t kTcCtrlBytes = 128;                   // mbarrier, TMEM address, flags
// 8 warps: warps w and w + 4 read the same 32 TMEM lanes (a warp reaches only
// its quarter) and take alternate 16-column chunks of the epilogue
constexpr int kTcThreads = 256;
// longest wait for the tensor cores to finish a patch before the kernel gives
// up (reported through g_cnn_tc_timeouts); a patch takes microseconds
constexpr uint64_t kTcWaitNs = 2000000000ull;

__device__ unsigned int g_cnn_tc_timeouts;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Shared-memory matrix descriptor, no swizzle: start, leading (K) and stride
// (M / N) byte offsets in 16-byte units, descriptor version 1 at bit 46.
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return uint64_t((saddr >> 4) & 0x3FFFu) | (uint64_t((lbo >> 4) & 0x3FFFu) << 16) |
         (uint64_t((sbo >> 4) & 0x3FFFu) << 32) | (uint64_t(1) << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), BF16 A
// and B (bits 7-9, 10-12 = 1), both K-major, N / 8 at bit 17, M / 16 at bit 24.
__host__ __device__ constexpr uint32_t tc_idesc(uint32_t m, uint32_t n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((m >> 4) << 24);
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n.reg .pred p;\n"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}

// Waits for phase `parity` of the barrier for at most kTcWaitNs.
__device__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity) {
  const uint64_t t0 = global_ns();
  for (;;) {
    if (mbar_try_wait(bar, parity)) return true;
    if (global_ns() - t0 > kTcWaitNs) return false;
  }
}

__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, bool valid) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src),
               "r"(valid ? 16 : 0)
               : "memory");
}

__global__ void __launch_bounds__(kTcThreads)
    conv3x3_tc_kernel(const ConvArgs a, uint32_t tmem_cols, int n_halos) {
  // n_halos halo buffers in a ring (1 to 4): the halos of the next n_halos - 1
  // patches are in flight while a patch's MMAs and epilogue run
  extern __shared__ __align__(128) unsigned char smem_tc[];
  const int cin = a.c1 + a.c2, kc_n = cin / 8, cout = a.cout;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem_tc);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem_tc + 8);
  int* flag = reinterpret_cast<int*>(smem_tc + 12);
  const uint32_t halo_bytes = uint32_t(kc_n) * kTcHR * kTcHC * 16;
  unsigned char* halo0 = smem_tc + kTcCtrlBytes;                 // n_halos x [kc][18][10][8]
  unsigned char* wsm = halo0 + size_t(n_halos) * halo_bytes;      // [9][kc][cout][8]
  const uint32_t bar_a = smem_addr(bar), halo_a = smem_addr(halo0), w_a = smem_addr(wsm);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int tiles_x = (a.w + kTcCols - 1) / kTcCols, tiles_y = (a.h + kTcRows - 1) / kTcRows;
  const int n_tiles = a.n * tiles_x * tiles_y;

  // the halo of patch t into halo buffer `buf`, 8 channels per 16-byte copy,
  // zero outside the image; one cp.async group per call (empty past the last patch)
  auto load_halo = [&](int t, int buf) {
    if (t >= n_tiles) {
      asm volatile("cp.async.commit_group;\n" ::: "memory");
      return;
    }
    const int img = t / (tiles_x * tiles_y);
    const int y0 = ((t / tiles_x) % tiles_y) * kTcRows - 1, x0 = (t % tiles_x) * kTcCols - 1;
    const uint32_t dst = halo_a + uint32_t(buf) * halo_bytes;
    constexpr int kPos = kTcHR * kTcHC;  // 180 halo pixels; a thread takes one or two
    const int kc1 = a.c1 / 8;
    for (int pos = tid; pos < kPos; pos += kTcThreads) {
      const int yy = y0 + pos / kTcHC, xx = x0 + pos % kTcHC;
      const bool in = yy >= 0 && yy < a.h && xx >= 0 && xx < a.w;
      // the pixel's channels are contiguous: one 16-byte copy per octet
      const __nv_bfloat16* s1 = a.x1 + (in ? x1_pixel(a, img, yy, xx) : 0) * a.c1;
      uint32_t d = dst + uint32_t(pos) * 16;
      for (int kc = 0; kc < kc1; ++kc, d += kPos * 16) cp_async16(d, s1 + kc * 8, in);
      if (kc1 < kc_n) {
        const __nv_bfloat16* s2 = a.x2 + (in ? (size_t(img) * a.h + yy) * a.w + xx : 0) * a.c2;
        for (int kc = 0; kc < kc_n - kc1; ++kc, d += kPos * 16) cp_async16(d, s2 + kc * 8, in);
      }
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
  };

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                     smem_addr(tmem_slot)),
                 "r"(tmem_cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar_a) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    *flag = 0;
  }
  // all taps' weights, re-laid from [tap][cout][cin] into core matrices, and
  // the first patch's halo
  for (int i = tid; i < 9 * kc_n * cout; i += kTcThreads) {
    const int co = i % cout, kc = (i / cout) % kc_n, tap = i / (cout * kc_n);
    cp_async16(w_a + uint32_t(i) * 16, a.wt + (size_t(tap) * cout + co) * cin + kc * 8, true);
  }
  asm volatile("cp.async.commit_group;\n" ::: "memory");
  const int stride = int(gridDim.x);
  for (int k = 0; k < max(1, n_halos - 1); ++k) load_halo(int(blockIdx.x) + k * stride, k);
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  const uint32_t idesc = tc_idesc(128, uint32_t(cout));
  constexpr uint32_t kLboA = kTcHR * kTcHC * 16, kSboA = kTcHC * 16;
  const uint32_t lbo_b = uint32_t(cout) * 16, sbo_b = 128;
  uint32_t phase = 0;
  bool ok = true;
  int k = 0;  // this CTA's patch counter: patch blockIdx.x + k * gridDim.x, buffer k % n_halos

  for (int t = blockIdx.x; t < n_tiles; t += stride, ++k) {
    const int buf = k % n_halos;
    if (n_halos >= 2) {
      // the ring's free buffer (patch k - 1's, whose MMAs are done) takes the
      // patch n_halos - 1 ahead; then patch k's group, the oldest, has landed
      load_halo(t + (n_halos - 1) * stride, (k + n_halos - 1) % n_halos);
      switch (n_halos) {
        case 2: asm volatile("cp.async.wait_group 1;\n" ::: "memory"); break;
        case 3: asm volatile("cp.async.wait_group 2;\n" ::: "memory"); break;
        default: asm volatile("cp.async.wait_group 3;\n" ::: "memory"); break;
      }
    } else {
      asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    }
    // make the copies visible to the tensor cores' (async proxy) reads
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      // The descriptors advance by adding to their start-address field (in
      // 16-byte units; every address is below 256 KB, so nothing carries out of
      // the field): A by one channel-octet pair per K step and by the tap's
      // (ky * 10 + kx) offset, B through the weights in order.
      const uint64_t a0 = tc_desc(halo_a + uint32_t(buf) * halo_bytes, kLboA, kSboA);
      uint64_t bd = tc_desc(w_a, lbo_b, sbo_b);
      const int ksteps = kc_n / 2;
      const uint64_t a_step = 2 * kTcHR * kTcHC, b_step = uint64_t(2 * cout);
      uint32_t acc = 0;
#pragma unroll
      for (int tap = 0; tap < 9; ++tap) {
        uint64_t ad = a0 + uint64_t((tap / 3) * kTcHC + tap % 3);
        for (int s = 0; s < ksteps; ++s) {
          asm volatile(
              "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
              "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
              "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
              : "memory");
          acc = 1;
          ad += a_step;
          bd += b_step;
        }
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
              bar_a)
          : "memory");
    }
    if (tid == 0 && !mbar_wait_bounded(bar_a, phase)) *flag = 1;
    __syncthreads();
    phase ^= 1u;
    if (*flag) {
      ok = false;
      break;
    }
    // with one buffer the next halo streams in under the epilogue (the MMAs
    // no longer read it)
    if (n_halos == 1) load_halo(t + stride, 0);
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    // epilogue: warps w and w + 4 hold TMEM lanes (pixels) 32w .. 32w + 31
    const int img = t / (tiles_x * tiles_y);
    const int ty = (t / tiles_x) % tiles_y, tx = t % tiles_x;
    const int quad = warp & 3, half = warp >> 2;
    const int m = quad * 32 + lane;
    const int oy = ty * kTcRows + m / kTcCols, ox = tx * kTcCols + m % kTcCols;
    const bool live = oy < a.h && ox < a.w;
    const size_t p = (size_t(img) * a.h + oy) * a.w + ox;
    for (int c0 = 16 * half; c0 < cout; c0 += 32) {
      float v[16];
      tc_ld16(tmem + (uint32_t(quad * 32) << 16) + uint32_t(c0), v);
      if (!live) continue;
#pragma unroll
      for (int e = 0; e < 16; ++e) {
        const int co = c0 + e;
        if (a.bias) v[e] += a.bias[co];
        if (a.slope >= 0.0f && v[e] < 0.0f) v[e] *= a.slope;
      }
      if (a.shuffle) {  // cout == 16: the whole 2 x 2 block of output pixels
#pragma unroll
        for (int sub = 0; sub < 4; ++sub) {
          const int yy = 2 * oy + (sub >> 1), xx = 2 * ox + (sub & 1);
          if (yy >= a.oh || xx >= a.ow) continue;
          float4* o = reinterpret_cast<float4*>(a.shuffle) + (size_t(img) * a.oh + yy) * a.ow + xx;
          float4 q = *o;
          q.x += v[sub];
          q.y += v[4 + sub];
          q.z += v[8 + sub];
          q.w += v[12 + sub];
          *o = q;
        }
        continue;
      }
      if (a.y_bf16) {
        uint32_t w8[8];
#pragma unroll
        for (int e = 0; e < 8; ++e)
          w8[e] = pack_bf16(__float2bfloat16_rn(v[2 * e]), __float2bfloat16_rn(v[2 * e + 1]));
        uint4* dst = reinterpret_cast<uint4*>(a.y_bf16 + p * cout + c0);
        dst[0] = make_uint4(w8[0], w8[1], w8[2], w8[3]);
        dst[1] = make_uint4(w8[4], w8[5], w8[6], w8[7]);
      }
      if (a.y_f32 && !a.y2_f32 && !a.accumulate) {  // plain FP32 output: 16-byte stores
        float4* dst = reinterpret_cast<float4*>(a.y_f32 + p * cout + c0);
#pragma unroll
        for (int e = 0; e < 4; ++e)
          dst[e] = make_float4(v[4 * e], v[4 * e + 1], v[4 * e + 2], v[4 * e + 3]);
        continue;
      }
#pragma unroll
      for (int e = 0; e < 16; ++e) {
        const int co = c0 + e;
        if (co < a.split) {
          if (a.y_f32) {
            float* o = a.y_f32 + p * a.split + co;
            *o = a.accumulate ? *o + v[e] : v[e];
          }
        } else if (a.y2_f32) {
          float* o = a.y2_f32 + p * (cout - a.split) + (co - a.split);
          *o = a.accumulate ? *o + v[e] : v[e];
        }
      }
    }
    // TMEM read before the next patch's MMAs overwrite it
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  }
  if (!ok && tid == 0) {
    atomicAdd(&g_cnn_tc_timeouts, 1u);
    mbar_wait_bounded(bar_a, phase ^ 1u);  // the abandoned patch's MMAs, bounded again
  }
  asm volatile("cp.async.wait_all;\n" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem),
                 "r"(tmem_cols)
                 : "memory");
  }
}

// ------------------------------------------------------------- weight gradient

struct WgradArgs {
  const __nv_bfloat16* x1;  // forward input (concatenation of x1, x2)
  const __nv_bfloat16* x2;
  int c1, c2;
  const __nv_bfloat16* gy;  // gradient at the pre-activation output [n][h][w][cout]
  int n, h, w, cout;
  float* dw;                // [9][cout][cin], accumulated
  float* db;                // [cout], accumulated (tap-0 CTAs only), or null
  int patches_per_cta;
};

// dW[tap][co][ci] = sum over pixels p of G[p][co] * X[p + tap][ci]: a GEMM with
// M = output channels, N = input channels and K = pixels.  CTA (tap, chunk)
// walks its chunk of 8x8 patches, staging G and the tap-shifted X in shared
// memory; warp w owns output channels 16w .. 16w+15 and all input channels.
template <int kNT>  // n-tiles of 8 input channels
__global__ void __launch_bounds__(kThreads) wgrad_kernel(const WgradArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int cin = a.c1 + a.c2;
  const int gpad = a.cout + 8, xpad = cin + 8;
  __nv_bfloat16* gs = reinterpret_cast<__nv_bfloat16*>(smem_raw);   // [64][gpad]
  __nv_bfloat16* xs = gs + 64 * gpad;                               // [64][xpad]
  const int tap = blockIdx.y, ky = tap / 3 - 1, kx = tap % 3 - 1;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int g = lane >> 2, q = lane & 3;
  const int tiles_x = (a.w + 7) / 8, tiles_y = (a.h + 7) / 8;
  const int n_patches = a.n * tiles_x * tiles_y;
  const int p_begin = blockIdx.x * a.patches_per_cta;
  const int p_end = min(n_patches, p_begin + a.patches_per_cta);
  const int m0 = warp * 16;
  const bool warp_active = m0 < a.cout;
  float acc[kNT][4];
#pragma unroll
  for (int j = 0; j < kNT; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
  float bacc = 0.0f;  // bias gradient of channel tid (tap-0 CTAs)
  for (int pt = p_begin; pt < p_end; ++pt) {
    const int img = pt / (tiles_x * tiles_y);
    const int tyy = (pt / tiles_x) % tiles_y, txx = pt % tiles_x;
    __syncthreads();
    for (int i = tid; i < 64 * a.cout; i += kThreads) {
      const int pix = i / a.cout, co = i % a.cout;
      const int yy = tyy * 8 + pix / 8, xx = txx * 8 + pix % 8;
      __nv_bfloat16 v = __float2bfloat16_rn(0.0f);
      if (yy < a.h && xx < a.w) v = a.gy[((size_t(img) * a.h + yy) * a.w + xx) * a.cout + co];
      gs[pix * gpad + co] = v;
    }
    for (int i = tid; i < 64 * cin; i += kThreads) {
      const int pix = i / cin, c = i % cin;
      const int yy = tyy * 8 + pix / 8 + ky, xx = txx * 8 + pix % 8 + kx;
      const int oy = tyy * 8 + pix / 8, ox = txx * 8 + pix % 8;
      __nv_bfloat16 v = __float2bfloat16_rn(0.0f);
      if (oy < a.h && ox < a.w && yy >= 0 && yy < a.h && xx >= 0 && xx < a.w) {
        const size_t p = (size_t(img) * a.h + yy) * a.w + xx;
        v = c < a.c1 ? a.x1[p * a.c1 + c] : a.x2[p * a.c2 + (c - a.c1)];
      }
      xs[pix * xpad + c] = v;
    }
    __syncthreads();
    if (a.db && tap == 4 && tid < a.cout)
      for (int pix = 0; pix < 64; ++pix) bacc += __bfloat162float(gs[pix * gpad + tid]);
    if (!warp_active) continue;
    for (int k0 = 0; k0 < 64; k0 += 16) {
      // A (16 x 16, m = output channel, k = pixel) from G^T
      uint32_t af[4];
      const int ma = m0 + g, mb = m0 + g + 8;
      const int ka = k0 + 2 * q, kb = k0 + 8 + 2 * q;
      auto gat = [&](int pix, int co) {
        return co < a.cout ? gs[pix * gpad + co] : __float2bfloat16_rn(0.0f);
      };
      af[0] = pack_bf16(gat(ka, ma), gat(ka + 1, ma));
      af[1] = pack_bf16(gat(ka, mb), gat(ka + 1, mb));
      af[2] = pack_bf16(gat(kb, ma), gat(kb + 1, ma));
      af[3] = pack_bf16(gat(kb, mb), gat(kb + 1, mb));
#pragma unroll
      for (int j = 0; j < kNT; ++j) {
        const int ci = j * 8 + g;
        const uint32_t b0 = pack_bf16(xs[ka * xpad + ci], xs[(ka + 1) * xpad + ci]);
        const uint32_t b1 = pack_bf16(xs[kb * xpad + ci], xs[(kb + 1) * xpad + ci]);
        mma_bf16(acc[j], af, b0, b1);
      }
    }
  }
  if (a.db && tap == 4 && tid < a.cout) atomicAdd(&a.db[tid], bacc);
  if (!warp_active) return;
#pragma unroll
  for (int j = 0; j < kNT; ++j) {
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int co = m0 + g + (e >= 2 ? 8 : 0);
      const int ci = j * 8 + 2 * q + (e & 1);
      if (co < a.cout && ci < cin)
        atomicAdd(&a.dw[(size_t(tap) * a.cout + co) * cin + ci], acc[j][e]);
    }
  }
}

// ------------------------------------------------------------- elementwise

// G = dY * LeakyReLU'(Y) (Y > 0 exactly when the pre-activation is), as BF16
__global__ void act_grad_kernel(const float* __restrict__ dy, const __nv_bfloat16* __restrict__ y,
                                float slope, __nv_bfloat16* __restrict__ gout, size_t n) {
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += size_t(gridDim.x) * blockDim.x) {
    const float d = dy[i];
    const float v = (!y || slope < 0.0f || __bfloat162float(y[i]) > 0.0f) ? d : d * slope;
    gout[i] = __float2bfloat16_rn(v);
  }
}

__global__ void avgpool2_kernel(const __nv_bfloat16* __restrict__ x, int n, int h, int w, int c,
                                __nv_bfloat16* __restrict__ y) {
  const int ho = h / 2, wo = w / 2;
  const size_t total = size_t(n) * ho * wo * c;
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
       i += size_t(gridDim.x) * blockDim.x) {
    const int ch = int(i % c);
    const size_t p = i / c;
    const int xo = int(p % wo), yo = int((p / wo) % ho), img = int(p / (size_t(wo) * ho));
    const size_t b = ((size_t(img) * h + 2 * yo) * w + 2 * xo) * c + ch;
    const float s = (__bfloat162float(x[b]) + __bfloat162float(x[b + c])) +
                    (__bfloat162float(x[b + size_t(w) * c]) +
                     __bfloat162float(x[b + size_t(w) * c + c]));
    y[i] = __float2bfloat16_rn(s * 0.25f);
  }
}

__global__ void avgpool2_backward_kernel(const float* __restrict__ dy, int n, int h, int w, int c,
                                         float* __restrict__ dx, int accumulate) {
  const size_t total = size_t(n) * h * w * c;
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
       i += size_t(gridDim.x) * blockDim.x) {
    const int ch = int(i % c);
    const size_t p = i / c;
    const int xx = int(p % w), yy = int((p / w) % h), img = int(p / (size_t(w) * h));
    const size_t o = ((size_t(img) * (h / 2) + yy / 2) * (w / 2) + xx / 2) * c + ch;
    const float v = dy[o] * 0.25f;
    dx[i] = accumulate ? dx[i] + v : v;
  }
}

// The same, eight channels (16 bytes) per thread; c8 = channels / 8.
__global__ void avgpool2_vec8_kernel(const uint4* __restrict__ x, int n, int h, int w, int c8,
                                     uint4* __restrict__ y) {
  const int ho = h / 2, wo = w / 2;
  const size_t total = size_t(n) * ho * wo * c8;
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
       i += size_t(gridDim.x) * blockDim.x) {
    const int ch = int(i % c8);
    const size_t p = i / c8;
    const int xo = int(p % wo), yo = int((p / wo) % ho), img = int(p / (size_t(wo) * ho));
    const size_t b = ((size_t(img) * h + 2 * yo) * w + 2 * xo) * c8 + ch;
    uint4 q[4] = {x[b], x[b + c8], x[b + size_t(w) * c8], x[b + size_t(w) * c8 + c8]};
    const __nv_bfloat16* e[4];
    for (int k = 0; k < 4; ++k) e[k] = reinterpret_cast<const __nv_bfloat16*>(&q[k]);
    uint4 r;
    uint32_t* rw = reinterpret_cast<uint32_t*>(&r);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      __nv_bfloat16 o[2];
#pragma unroll
      for (int t = 0; t < 2; ++t) {
        const int k = 2 * j + t;
        const float s = (__bfloat162float(e[0][k]) + __bfloat162float(e[1][k])) +
                        (__bfloat162float(e[2][k]) + __bfloat162float(e[3][k]));
        o[t] = __float2bfloat16_rn(s * 0.25f);
      }
      rw[j] = pack_bf16(o[0], o[1]);
    }
    y[i] = r;
  }
}

__global__ void upsample2_kernel(const __nv_bfloat16* __restrict__ x, int n, int h, int w, int c,
                                 __nv_bfloat16* __restrict__ y) {
  const size_t total = size_t(n) * (2 * h) * (2 * w) * c;
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
       i += size_t(gridDim.x) * blockDim.x) {
    const int ch = int(i % c);
    const size_t p = i / c;
    const int xx = int(p % (2 * w)), yy = int((p / (2 * w)) % (2 * h));
    const int img = int(p / (size_t(4) * w * h));
    y[i] = x[((size_t(img) * h + yy / 2) * w + xx / 2) * c + ch];
  }
}

__global__ void upsample2_backward_kernel(const float* __restrict__ dy, int n, int h, int w, int c,
                                          float* __restrict__ dx) {
  const size_t total = size_t(n) * h * w * c;
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
       i += size_t(gridDim.x) * blockDim.x) {
    const int ch = int(i % c);
    const size_t p = i / c;
    const int xx = int(p % w), yy = int((p / w) % h), img = int(p / (size_t(w) * h));
    const size_t b = ((size_t(img) * 2 * h + 2 * yy) * 2 * w + 2 * xx) * c + ch;
    const size_t r = size_t(2 * w) * c;
    dx[i] = (dy[b] + dy[b + c]) + (dy[b + r] + dy[b + r + c]);
  }
}

// out[Y][X][ch] = base[Y][X][ch] + head[Y/2][X/2][ch*4 + (Y%2)*2 + X%2] (pixel
// shuffle) for the oh x ow output (at most 2h x 2w); base and out may alias
__global__ void head_kernel(const float* __restrict__ head, const float* base, int n, int h, int w,
                            int oh, int ow, float* out) {
  const size_t total = size_t(n) * oh * ow * 4;
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
       i += size_t(gridDim.x) * blockDim.x) {
    const int ch = int(i & 3);
    const size_t p = i >> 2;
    const int xx = int(p % ow), yy = int((p / ow) % oh);
    const int img = int(p / (size_t(ow) * oh));
    const int sub = ch * 4 + (yy & 1) * 2 + (xx & 1);
    out[i] = base[i] + head[((size_t(img) * h + yy / 2) * w + xx / 2) * 16 + sub];
  }
}

// Network input of a reduced frame: RGBA of the w x h image in channels 0..3,
// zero elsewhere and in the padding up to wp x hp, as BF16 [hp][wp][16]
__global__ void prepare_input_kernel(const float4* __restrict__ img,
                                     const float* __restrict__ depth, int h, int w, int hp, int wp,
                                     uint32_t* __restrict__ out) {
  const size_t total = size_t(hp) * wp * 8;  // 8 words (16 BF16) per pixel
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
       i += size_t(gridDim.x) * blockDim.x) {
    const int word = int(i & 7);
    const size_t p = i >> 3;
    const int xx = int(p % wp), yy = int(p / wp);
    uint32_t v = 0;
    if (word < 2 && xx < w && yy < h) {
      const float4 c = img[size_t(yy) * w + xx];
      v = word == 0 ? pack_bf16(__float2bfloat16_rn(c.x), __float2bfloat16_rn(c.y))
                    : pack_bf16(__float2bfloat16_rn(c.z), __float2bfloat16_rn(c.w));
    } else if (word == 2 && depth && xx < w && yy < h) {
      v = pack_bf16(__float2bfloat16_rn(depth[size_t(yy) * w + xx]), __float2bfloat16_rn(0.0f));
    }
    out[i] = v;
  }
}

// Mean squared RGBA difference between the probe rays and the same pixels of a
// frame: probe pixel (x, y) is frame pixel (x * stride + ox, y * stride + oy).
__global__ void probe_mse_kernel(const float4* __restrict__ frame, int w,
                                 const float4* __restrict__ probe, int pw, int ph, int stride,
                                 int ox, int oy, float* __restrict__ sum) {
  float s = 0.0f;
  const int n = pw * ph;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int x = i % pw, y = i / pw;
    const float4 a = frame[size_t(y * stride + oy) * w + x * stride + ox];
    const float4 b = probe[i];
    const float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z, dw = a.w - b.w;
    s += (dx * dx + dy * dy) + (dz * dz + dw * dw);
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(sum, s);
}

__global__ void head_backward_kernel(const float* __restrict__ dout, int n, int h, int w,
                                     float* __restrict__ dhead) {
  const size_t total = size_t(n) * h * w * 16;
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
       i += size_t(gridDim.x) * blockDim.x) {
    const int sub = int(i & 15);
    const size_t p = i >> 4;
    const int xx = int(p % w), yy = int((p / w) % h), img = int(p / (size_t(w) * h));
    const int ch = sub >> 2, dyy = (sub >> 1) & 1, dxx = sub & 1;
    dhead[i] = dout[((size_t(img) * 2 * h + 2 * yy + dyy) * 2 * w + 2 * xx + dxx) * 4 + ch];
  }
}

// mean squared error over all elements: loss accumulated into *loss (sum of
// squares / n), gradient 2 (out - target) / n
__global__ void mse_kernel(const float* __restrict__ out, const float* __restrict__ target,
                           size_t n, float* __restrict__ dout, float* __restrict__ loss) {
  float s = 0.0f;
  const float inv = 1.0f / float(n);
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += size_t(gridDim.x) * blockDim.x) {
    const float d = out[i] - target[i];
    if (dout) dout[i] = 2.0f * d * inv;
    s += d * d;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, s * inv);
}

// Adam on the FP32 masters, then the BF16 copies: forward [tap][cout][cin]
// and backward-data [8 - tap][cin][cout] (flipped taps, swapped channels)
__global__ void adam_kernel(float* __restrict__ w, const float* __restrict__ g,
                            float* __restrict__ m, float* __restrict__ v, size_t n, float lr,
                            float b1, float b2, float eps, float c1, float c2) {
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += size_t(gridDim.x) * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

__global__ void weights_bf16_kernel(const float* __restrict__ w, int cout, int cin,
                                    __nv_bfloat16* __restrict__ fwd,
                                    __nv_bfloat16* __restrict__ bwd) {
  const size_t total = size_t(9) * cout * cin;
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
       i += size_t(gridDim.x) * blockDim.x) {
    const int ci = int(i % cin), co = int((i / cin) % cout), tap = int(i / (size_t(cin) * cout));
    const __nv_bfloat16 b = __float2bfloat16_rn(w[i]);
    fwd[i] = b;
    if (bwd) bwd[(size_t(8 - tap) * cin + ci) * cout + co] = b;
  }
}

__global__ void to_bf16_kernel(const float* __restrict__ x, size_t n, __nv_bfloat16* __restrict__ y) {
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += size_t(gridDim.x) * blockDim.x)
    y[i] = __float2bfloat16_rn(x[i]);
}

uint32_t grid_for(size_t n) {
  const size_t b = (n + 255) / 256;
  return uint32_t(b < 152 * 32 ? (b ? b : 1) : 152 * 32);
}

// Shared memory of conv3x3_tc_kernel: control words, a ring of halos, the
// weights.  Every MMA descriptor stays inside its operand: the A operand of
// the last K step of tap (2, 2) ends at ((2 (kc/2 - 1) * 18 + 2) * 10 + 2) * 16
// + 2880 + 15 * 160 + 128 <= kc * 2880 bytes, and B's at the end of the weights.
size_t conv_tc_smem(int cin, int cout, int n_halos) {
  const size_t kc = size_t(cin) / 8;
  return kTcCtrlBytes + size_t(n_halos) * kc * kTcHR * kTcHC * 16 + 9 * kc * size_t(cout) * 16;
}

// The tcgen05 convolution takes the launch when its shapes fit: input and
// output channels multiples of 16 (M = 128, N = cout, K steps of 16), at most
// 128 output channels (a power-of-two TMEM allocation of 32 to 128 columns),
// 16-byte aligned tensors, and halo + weights in shared memory.
bool launch_conv_tc(const ConvArgs& a, cudaStream_t s) {
  const int cin = a.c1 + a.c2;
  auto aligned = [](const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; };
  if (cin % 16 || a.c1 % 8 || a.c2 % 8 || cin > 128) return false;
  if (a.cout % 16 || a.cout < 16 || a.cout > 128) return false;
  if (!aligned(a.x1) || (a.c2 && !aligned(a.x2)) || !aligned(a.wt) || !aligned(a.y_bf16) ||
      !aligned(a.y_f32))
    return false;
  constexpr size_t kMaxSmem = 227 * 1024, kSmPerSm = 228 * 1024, kReserved = 1024;
  const uint32_t cols = a.cout <= 32 ? 32u : a.cout <= 64 ? 64u : 128u;
  // CTAs per SM that tensor memory (512 columns), threads and registers allow
  static int regs = 0;
  if (!regs) {
    cudaFuncAttributes fa{};
    TVK_CUDA(cudaFuncGetAttributes(&fa, conv3x3_tc_kernel));
    regs = std::max(1, fa.numRegs);
  }
  const int max_ctas = std::max(1, std::min({int(512 / cols), 2048 / kTcThreads,
                                             65536 / (regs * kTcThreads)}));
  // CTAs per SM and halos per CTA (each CTA also reserves 1 KB of shared
  // memory): the most CTAs whose shares hold 2 halos each (the next patch's
  // input streaming in under the MMAs), when that is at least 3; otherwise the
  // most CTAs that hold one.  Each CTA takes the deepest ring (up to 4) its
  // share holds.  Measured on the network's layers at 960x540: 80 -> 32
  // channels 85 us with 3 CTAs of one halo against 105 us with 2 of two; 16 ->
  // 32 channels 51 us with 10 CTAs of two against 56 us with 13 of one.
  const size_t halo = size_t(cin) / 8 * kTcHR * kTcHC * 16;
  const size_t base = conv_tc_smem(cin, a.cout, 0);
  auto ring = [&](int c) {
    const size_t per = kSmPerSm / size_t(c) - kReserved;
    const size_t room = std::min(per, kMaxSmem);
    return room > base ? int(std::min<size_t>((room - base) / halo, 4)) : 0;
  };
  auto most_ctas = [&](int min_halos) {
    for (int c = max_ctas; c >= 1; --c)
      if (ring(c) >= min_halos) return c;
    return 0;
  };
  int per_sm = most_ctas(2);
  if (per_sm < 3) per_sm = std::max(most_ctas(1), 1);
  const int n_halos = ring(per_sm);
  if (n_halos < 1) return false;
  const size_t smem = conv_tc_smem(cin, a.cout, n_halos);
  // once per device: the kernel's shared-memory limit and carveout, and the SM
  // count (host calls between the network's short launches would leave the
  // GPU waiting)
  int dev = 0;
  TVK_CUDA(cudaGetDevice(&dev));
  static std::mutex mu;
  static int sms_of[64] = {0};
  int sms = 0;
  {
    std::lock_guard<std::mutex> lock(mu);
    if (dev < 0 || dev >= 64) fail(TVK_ERR_INTERNAL, "device ordinal out of range");
    if (!sms_of[dev]) {
      TVK_CUDA(cudaFuncSetAttribute(conv3x3_tc_kernel,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    int(kMaxSmem)));
      TVK_CUDA(cudaFuncSetAttribute(conv3x3_tc_kernel,
                                    cudaFuncAttributePreferredSharedMemoryCarveout,
                                    int(cudaSharedmemCarveoutMaxShared)));
      TVK_CUDA(cudaDeviceGetAttribute(&sms_of[dev], cudaDevAttrMultiProcessorCount, dev));
    }
    sms = sms_of[dev];
  }
  // a persistent grid of the CTAs that fit on an SM together; resident CTAs
  // never wait on one another for tensor memory (512 columns)
  const long tiles = long(a.n) * ((a.w + kTcCols - 1) / kTcCols) * ((a.h + kTcRows - 1) / kTcRows);
  const unsigned grid = unsigned(std::min<long>(tiles, long(per_sm) * sms));
  conv3x3_tc_kernel<<<grid, kTcThreads, smem, s>>>(a, cols, n_halos);
  TVK_CUDA(cudaGetLastError());
  return true;
}

}  // namespace

void cnn_conv3x3_shuffle(const CnnConv& c, float* out, int oh, int ow, cudaStream_t s) {
  ConvArgs a{};
  a.x1 = static_cast<const __nv_bfloat16*>(c.x1);
  a.c1 = c.c1;
  a.n = c.n;
  a.h = c.h;
  a.w = c.w;
  a.wt = static_cast<const __nv_bfloat16*>(c.weights);
  a.bias = c.bias;
  a.cout = c.cout;
  a.slope = c.slope;
  a.split = c.cout;
  a.shuffle = out;
  a.oh = oh;
  a.ow = ow;
  if (c.cout == 16 && c.c2 == 0 && !c.upsample1 &&
      (reinterpret_cast<uintptr_t>(out) & 15u) == 0 && launch_conv_tc(a, s))
    return;
  // other shapes: the FP32 convolution, then the shuffle as its own pass
  if (!c.y_f32) fail(TVK_ERR_INTERNAL, "shuffle convolution without a fallback buffer");
  cnn_conv3x3(c, s);
  cnn_head(c.y_f32, out, c.n, c.h, c.w, oh, ow, out, s);
}

uint32_t cnn_tc_timeouts(bool reset) {
  uint32_t n = 0;
  TVK_CUDA(cudaMemcpyFromSymbol(&n, g_cnn_tc_timeouts, sizeof(n)));
  if (reset && n) {
    const uint32_t zero = 0;
    TVK_CUDA(cudaMemcpyToSymbol(g_cnn_tc_timeouts, &zero, sizeof(zero)));
  }
  return n;
}

void cnn_conv3x3(const CnnConv& c, cudaStream_t s) {
  ConvArgs a{};
  a.x1 = static_cast<const __nv_bfloat16*>(c.x1);
  a.x2 = static_cast<const __nv_bfloat16*>(c.x2);
  a.c1 = c.c1;
  a.c2 = c.c2;
  a.n = c.n;
  a.h = c.h;
  a.w = c.w;
  a.wt = static_cast<const __nv_bfloat16*>(c.weights);
  a.bias = c.bias;
  a.cout = c.cout;
  a.slope = c.slope;
  a.y_bf16 = static_cast<__nv_bfloat16*>(c.y_bf16);
  a.y_f32 = c.y_f32;
  a.y2_f32 = c.y2_f32;
  a.split = c.y2_f32 ? c.split : c.cout;
  a.accumulate = c.accumulate;
  a.up1 = c.upsample1 ? 1 : 0;
  a.h1 = c.h1;
  a.w1 = c.w1;
  const int cin = c.c1 + c.c2;
  const int nt = (c.cout + 7) / 8;
  if (launch_conv_tc(a, s)) return;
  // large images: 16x16 patches (all taps' weights staged when they fit in
  // 64 KB with the halo), while there are at least two waves of them
  const unsigned wide_blocks =
      unsigned(c.n) * ((c.w + kWideTile - 1) / kWideTile) * ((c.h + kWideTile - 1) / kWideTile);
  if (wide_blocks >= 2 * 152 && nt <= 8) {
    const size_t pitch = size_t(cin + 8) * sizeof(__nv_bfloat16);
    const size_t halo = size_t(kWideHalo) * kWideHalo * pitch;
    const size_t all = halo + size_t(9) * nt * 8 * pitch, one = halo + size_t(nt) * 8 * pitch;
    const bool all_taps = all <= 64 * 1024;
    const size_t smem = all_taps ? all : one;
#define TVK_WIDE_CASE(NT)                                                                   \
  case NT:                                                                                  \
    if (all_taps) {                                                                         \
      TVK_CUDA(cudaFuncSetAttribute(conv3x3_wide_kernel<NT, true>,                          \
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem))); \
      conv3x3_wide_kernel<NT, true><<<wide_blocks, kWideThreads, smem, s>>>(a);             \
    } else {                                                                                \
      TVK_CUDA(cudaFuncSetAttribute(conv3x3_wide_kernel<NT, false>,                         \
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem))); \
      conv3x3_wide_kernel<NT, false><<<wide_blocks, kWideThreads, smem, s>>>(a);            \
    }                                                                                       \
    break;
    switch (nt) {
      TVK_WIDE_CASE(1)
      TVK_WIDE_CASE(2)
      TVK_WIDE_CASE(4)
      TVK_WIDE_CASE(6)
      TVK_WIDE_CASE(8)
      default: fail(TVK_ERR_UNSUPPORTED, "output channels must be 8, 16, 32, ..., 128");
    }
#undef TVK_WIDE_CASE
    TVK_CUDA(cudaGetLastError());
    return;
  }
  const size_t smem = (size_t(100) + size_t(nt) * 8) * (cin + 8) * sizeof(__nv_bfloat16);
  const unsigned blocks = unsigned(c.n) * ((c.w + 7) / 8) * ((c.h + 7) / 8);
#define TVK_CONV_CASE(NT)                                                                 \
  case NT:                                                                                \
    TVK_CUDA(cudaFuncSetAttribute(conv3x3_kernel<NT>,                                     \
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem))); \
    conv3x3_kernel<NT><<<blocks, kThreads, smem, s>>>(a);                                 \
    break;
  switch (nt) {
    TVK_CONV_CASE(1)
    TVK_CONV_CASE(2)
    TVK_CONV_CASE(4)
    TVK_CONV_CASE(6)
    TVK_CONV_CASE(8)
    TVK_CONV_CASE(10)
    TVK_CONV_CASE(12)
    TVK_CONV_CASE(14)
    TVK_CONV_CASE(16)
    default: fail(TVK_ERR_UNSUPPORTED, "output channels must be 8, 16, 32, ..., 128");
  }
#undef TVK_CONV_CASE
  TVK_CUDA(cudaGetLastError());
}

void cnn_conv3x3_wgrad(const CnnWgrad& c, cudaStream_t s) {
  WgradArgs a{};
  a.x1 = static_cast<const __nv_bfloat16*>(c.x1);
  a.x2 = static_cast<const __nv_bfloat16*>(c.x2);
  a.c1 = c.c1;
  a.c2 = c.c2;
  a.gy = static_cast<const __nv_bfloat16*>(c.gy);
  a.n = c.n;
  a.h = c.h;
  a.w = c.w;
  a.cout = c.cout;
  a.dw = c.dw;
  a.db = c.db;
  const int cin = c.c1 + c.c2;
  const int patches = c.n * ((c.w + 7) / 8) * ((c.h + 7) / 8);
  // about 4 CTAs per SM over the 9 taps
  const int chunks = std::max(1, std::min(patches, (152 * 4 + 8) / 9));
  a.patches_per_cta = (patches + chunks - 1) / chunks;
  const dim3 grid((patches + a.patches_per_cta - 1) / a.patches_per_cta, 9);
  const size_t smem = (size_t(64) * (c.cout + 8) + size_t(64) * (cin + 8)) * sizeof(__nv_bfloat16);
  const int nt = cin / 8;
#define TVK_WG_CASE(NT)                                                                   \
  case NT:                                                                                \
    TVK_CUDA(cudaFuncSetAttribute(wgrad_kernel<NT>,                                       \
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem))); \
    wgrad_kernel<NT><<<grid, kThreads, smem, s>>>(a);                                     \
    break;
  switch (nt) {
    TVK_WG_CASE(2)
    TVK_WG_CASE(4)
    TVK_WG_CASE(6)
    TVK_WG_CASE(8)
    TVK_WG_CASE(10)
    TVK_WG_CASE(12)
    TVK_WG_CASE(14)
    TVK_WG_CASE(16)
    default: fail(TVK_ERR_UNSUPPORTED, "input channels must be 16, 32, ..., 128");
  }
#undef TVK_WG_CASE
  TVK_CUDA(cudaGetLastError());
}

void cnn_act_grad(const float* dy, const void* y, float slope, void* g, size_t n, cudaStream_t s) {
  act_grad_kernel<<<grid_for(n), 256, 0, s>>>(dy, static_cast<const __nv_bfloat16*>(y), slope,
                                              static_cast<__nv_bfloat16*>(g), n);
  TVK_CUDA(cudaGetLastError());
}

void cnn_avgpool2(const void* x, int n, int h, int w, int c, void* y, cudaStream_t s) {
  const bool vec = c % 8 == 0 && (reinterpret_cast<uintptr_t>(x) & 15u) == 0 &&
                   (reinterpret_cast<uintptr_t>(y) & 15u) == 0;
  if (vec) {
    avgpool2_vec8_kernel<<<grid_for(size_t(n) * (h / 2) * (w / 2) * (c / 8)), 256, 0, s>>>(
        static_cast<const uint4*>(x), n, h, w, c / 8, static_cast<uint4*>(y));
  } else {
    avgpool2_kernel<<<grid_for(size_t(n) * (h / 2) * (w / 2) * c), 256, 0, s>>>(
        static_cast<const __nv_bfloat16*>(x), n, h, w, c, static_cast<__nv_bfloat16*>(y));
  }
  TVK_CUDA(cudaGetLastError());
}

void cnn_avgpool2_backward(const float* dy, int n, int h, int w, int c, float* dx, int accumulate,
                           cudaStream_t s) {
  avgpool2_backward_kernel<<<grid_for(size_t(n) * h * w * c), 256, 0, s>>>(dy, n, h, w, c, dx,
                                                                          accumulate);
  TVK_CUDA(cudaGetLastError());
}

void cnn_upsample2(const void* x, int n, int h, int w, int c, void* y, cudaStream_t s) {
  upsample2_kernel<<<grid_for(size_t(n) * 4 * h * w * c), 256, 0, s>>>(
      static_cast<const __nv_bfloat16*>(x), n, h, w, c, static_cast<__nv_bfloat16*>(y));
  TVK_CUDA(cudaGetLastError());
}

void cnn_upsample2_backward(const float* dy, int n, int h, int w, int c, float* dx,
                            cudaStream_t s) {
  upsample2_backward_kernel<<<grid_for(size_t(n) * h * w * c), 256, 0, s>>>(dy, n, h, w, c, dx);
  TVK_CUDA(cudaGetLastError());
}

void cnn_head(const float* head, const float* base, int n, int h, int w, int oh, int ow,
              float* out, cudaStream_t s) {
  head_kernel<<<grid_for(size_t(n) * 4 * oh * ow), 256, 0, s>>>(head, base, n, h, w, oh, ow, out);
  TVK_CUDA(cudaGetLastError());
}

void cnn_prepare_input(const float* img, const float* depth, int h, int w, int hp, int wp,
                       void* out, cudaStream_t s) {
  prepare_input_kernel<<<grid_for(size_t(hp) * wp * 8), 256, 0, s>>>(
      reinterpret_cast<const float4*>(img), depth, h, w, hp, wp, static_cast<uint32_t*>(out));
  TVK_CUDA(cudaGetLastError());
}

void cnn_probe_mse(const float* frame, int w, const float* probe, int pw, int ph, int stride,
                   int ox, int oy, float* sum, cudaStream_t s) {
  probe_mse_kernel<<<std::max(1, std::min(152 * 4, (pw * ph + 255) / 256)), 256, 0, s>>>(
      reinterpret_cast<const float4*>(frame), w, reinterpret_cast<const float4*>(probe), pw, ph,
      stride, ox, oy, sum);
  TVK_CUDA(cudaGetLastError());
}

void cnn_head_backward(const float* dout, int n, int h, int w, float* dhead, cudaStream_t s) {
  head_backward_kernel<<<grid_for(size_t(n) * 16 * h * w), 256, 0, s>>>(dout, n, h, w, dhead);
  TVK_CUDA(cudaGetLastError());
}

void cnn_mse(const float* out, const float* target, size_t n, float* dout, float* loss,
             cudaStream_t s) {
  mse_kernel<<<std::min<uint32_t>(grid_for(n), 152 * 8), 256, 0, s>>>(out, target, n, dout, loss);
  TVK_CUDA(cudaGetLastError());
}

void cnn_adam(float* w, const float* g, float* m, float* v, size_t n, float lr, float b1, float b2,
              float eps, int step, cudaStream_t s) {
  const float c1 = 1.0f - powf(b1, float(step)), c2 = 1.0f - powf(b2, float(step));
  adam_kernel<<<grid_for(n), 256, 0, s>>>(w, g, m, v, n, lr, b1, b2, eps, c1, c2);
  TVK_CUDA(cudaGetLastError());
}

void cnn_weights_bf16(const float* w, int cout, int cin, void* fwd, void* bwd, cudaStream_t s) {
  weights_bf16_kernel<<<grid_for(size_t(9) * cout * cin), 256, 0, s>>>(
      w, cout, cin, static_cast<__nv_bfloat16*>(fwd), static_cast<__nv_bfloat16*>(bwd));
  TVK_CUDA(cudaGetLastError());
}

void cnn_to_bf16(const float* x, size_t n, void* y, cudaStream_t s) {
  to_bf16_kernel<<<grid_for(n), 256, 0, s>>>(x, n, static_cast<__nv_bfloat16*>(y));
  TVK_CUDA(cudaGetLastError());
}

}  // namespace tvk
