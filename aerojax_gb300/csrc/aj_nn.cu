// Learned pressure warm start: a 4-level convolutional encoder-decoder on the
// tensor cores (BF16 operands, FP32 accumulation), its backward pass, MSE
// loss and Adam - the network, training and inference kernels.
//
// The reference's learned operators (neural_operators/nn_pressure_operator_*.py)
// replace the pressure solve; here the network predicts a correction to the
// previous pressure on a grid F times coarser, and the converging multigrid
// always finishes the solve.  Architecture (oracle/nn_np.py holds the same
// table): e0a 16->32, e0b 32->32 (s0) | pool | e1a 32->64, e1b 64->64 (s1) |
// pool | e2a 64->128, e2b 128->128 (s2) | pool | e3a, e3b 128->128 |
// up + s2 | d2 128->64 | up + s1 | d1 64->32 | up + s0 | d0a 32->32 |
// d0b 32->16 (linear; channel 0 is the prediction).  3x3 'SAME' convolutions
// (zero padding, bias, ReLU), 2x2 average pooling, nearest 2x upsampling.
// Activations are FP32 NHWC [n][h][w][c]; weights are kept as an FP32 master
// copy (flat: per layer W[3][3][Cin][Cout] then b[Cout]) and packed to BF16
// twice per layer: WfT[tap][Cout][Cin] for the forward pass and
// WbT[8-tap][Cin][Cout] (the adjoint of a stride-1 'SAME' convolution is the
// convolution with the flipped, channel-transposed kernel) for the input
// gradient.
#include "aj_internal.cuh"
#include <cuda_bf16.h>
#include <stdlib.h>
#include <string.h>

namespace aj {

struct NnLayer {
  int cin, cout, relu;
};
static const NnLayer kLayers[] = {
    {16, 32, 1}, {32, 32, 1}, {32, 64, 1}, {64, 64, 1}, {64, 128, 1}, {128, 128, 1},
    {128, 128, 1}, {128, 128, 1}, {128, 64, 1}, {64, 32, 1}, {32, 32, 1}, {32, 16, 0}};
enum { E0A, E0B, E1A, E1B, E2A, E2B, E3A, E3B, D2, D1, D0A, D0B, NL };

static size_t w_off(int l) {   // FP32 master offset of layer l's weights
  size_t o = 0;
  for (int k = 0; k < l; ++k) o += 9 * (size_t)kLayers[k].cin * kLayers[k].cout + kLayers[k].cout;
  return o;
}
static size_t b_off(int l) { return w_off(l) + 9 * (size_t)kLayers[l].cin * kLayers[l].cout; }
static size_t pk_off(int l) {  // packed BF16 offset of layer l (Wf then Wb)
  size_t o = 0;
  for (int k = 0; k < l; ++k) o += 2 * 9 * (size_t)kLayers[k].cin * kLayers[k].cout;
  return o;
}
static size_t n_params() { return w_off(NL); }
static size_t n_packed() { return pk_off(NL); }

// ---------------------------------------------------------------- MMA helpers
__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}

// D = A (16x16 bf16, row) * B (16x8 bf16, col) + D (f32)
__device__ __forceinline__ void mma_bf16(float* d, const uint32_t* a, const uint32_t* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// four 8x8 BF16 matrices from shared memory, one row address per lane
__device__ __forceinline__ void ldsm_x4(uint32_t* r, unsigned addr) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(addr));
}

// ---------------------------------------------------------------- convolution
// Implicit GEMM on 8 x 8 pixel tiles: M = 64 pixels (16 per warp: two tile
// rows), N = BN output channels of the block, K = 9 taps x Cin.  The block
// stages the BF16 weights of all 9 taps for its BN channels (WT[tap][co][ci])
// with cp.async and the 10 x 10 x Cin halo of its tile (zero-filled outside
// the image), rounded once to BF16 as it is stored; one barrier, then the
// whole K loop runs from shared memory, every tap an offset into the halo,
// the fragments loaded by ldmatrix.  Row strides of Cin + 8 BF16 keep the
// ldmatrix rows 16-byte aligned and free of bank conflicts.
constexpr int CT = 8;                       // pixel tile edge
constexpr int CT_HALO = (CT + 2) * (CT + 2);
constexpr int CONV_THREADS = 256;   // 8 warps: 4 pixel-row pairs x 2 halves of K

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int NPEND>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(NPEND));
}

template <int CIN, int NT>
struct ConvSmem {
  static constexpr int AS = CIN + 8, BN = NT * 8;   // BF16 row stride of the halo and the weights
  static constexpr size_t a_bytes = (size_t)CT_HALO * AS * 2;
  static constexpr size_t bytes = a_bytes + (size_t)9 * BN * AS * 2;
  static_assert(a_bytes % 16 == 0 && (AS * 2) % 16 == 0, "ldmatrix rows must be 16-byte aligned");
  static_assert((size_t)4 * NT * 4 * 32 * 4 <= bytes, "the K halves' hand-over must fit");
};

// One convolution's operands (NHWC activations, WT[tap][Cout][Cin] BF16).
struct ConvArgs {
  const float* X;
  int N, H, W, Cout;
  const __nv_bfloat16* WT;
  const float* bias;
  float* Y;
  int relu;
  float* Yp;         // nullable: 2x2 average pool of Y
  const float* Xc;   // nullable: the input is up2(Xc) + X
  const DevScalars* norm;   // nullable: scale input channels 0 and 2 by 1 / the
                            // sample's RMS (the features' normalisation)
};

// The output side of one conv tile: outputs of one 8 x 8 pixel tile and
// BN = NT * 8 channels from co0.
struct ConvOut {
  float* Y;
  float* Yp;          // nullable: 2x2 average pool of Y
  const float* bias;  // nullable
  int relu, H, W, Cout, n, h0, w0, co0;
};

// The K loop and epilogue of one conv tile from shared memory: As holds the
// tile's 10 x 10 halo in BF16 ([px][CIN + 8]), Bs the 9 taps' weights
// ([tap][BN][CIN + 8]); sm is the start of the block's dynamic shared memory
// (the K halves' hand-over buffer once the loop is done).
template <int CIN, int NT>
__device__ __forceinline__ void conv_core(const __nv_bfloat16* As, const __nv_bfloat16* Bs,
                                          unsigned char* sm, const ConvOut& o) {
  constexpr int AS = CIN + 8, BN = NT * 8;
  // two accumulator sets, even and odd 16-channel steps, halve each chain of
  // dependent MMAs again; they are added before the hand-over
  float acc[NT][4], acc2[NT][4];
#pragma unroll
  for (int q = 0; q < NT; ++q)
#pragma unroll
    for (int e = 0; e < 4; ++e) acc[q][e] = acc2[q][e] = 0.f;
  // warp w: tile rows 2 (w & 3) and 2 (w & 3) + 1 (fragment rows g, g + 8);
  // warps 0-3 run taps 0-4 and warps 4-7 taps 5-8, which halves each chain
  // of dependent MMAs (9 Cin / 16 of them in one warp before).  Fragments
  // come by ldmatrix: lane l addresses row l & 7 of 8x8 matrix l >> 3 - for
  // A the pixel (tile row + (m & 1), column r + dx) at channel offset
  // (m >> 1) * 8, for B output channel 8 (m >> 1) + r of the pair of
  // 8-channel groups at channel offset (m & 1) * 8.
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int g = lane >> 2, tg = lane & 3;
  float* __restrict__ Y = o.Y;
  float* __restrict__ Yp = o.Yp;
  const float* __restrict__ bias = o.bias;
  const int relu = o.relu, H = o.H, W = o.W, Cout = o.Cout, n = o.n, h0 = o.h0, w0 = o.w0,
            co0 = o.co0;
  const int prow = warp & 3, kh = warp >> 2;
  const int ty0 = 2 * prow;
  const int lm = lane >> 3, lr = lane & 7;
  const unsigned as0 = (unsigned)__cvta_generic_to_shared(As);
  const unsigned bs0 = (unsigned)__cvta_generic_to_shared(Bs);
  static_assert(NT % 2 == 0, "B fragments load in pairs of 8-channel groups");
#pragma unroll 1
  for (int tap = kh ? 5 : 0; tap < (kh ? 9 : 5); ++tap) {
    const int dy = tap / 3, dx = tap % 3;   // halo offsets (tap - centre + 1)
    const unsigned a_row =
        as0 + (unsigned)((((ty0 + dy + (lm & 1)) * (CT + 2) + lr + dx) * AS + (lm >> 1) * 8) * 2);
    const unsigned b_row = bs0 + (unsigned)(((tap * BN + (lm >> 1) * 8 + lr) * AS + (lm & 1) * 8) * 2);
#pragma unroll
    for (int ks = 0; ks < CIN / 16; ++ks) {
      uint32_t a[4];
      ldsm_x4(a, a_row + ks * 32);
#pragma unroll
      for (int qp = 0; qp < NT / 2; ++qp) {
        uint32_t b[4];
        ldsm_x4(b, b_row + (unsigned)(qp * 16 * AS * 2) + ks * 32);
        mma_bf16((ks & 1) ? acc2[2 * qp] : acc[2 * qp], a, b);
        mma_bf16((ks & 1) ? acc2[2 * qp + 1] : acc[2 * qp + 1], a, b + 2);
      }
    }
  }
#pragma unroll
  for (int q = 0; q < NT; ++q)
#pragma unroll
    for (int e = 0; e < 4; ++e) acc[q][e] += acc2[q][e];
  // warps 4-7 hand their partial sums to warps 0-3 through the (now free)
  // halo buffer; the sum is (taps 0-4) + (taps 5-8)
  __syncthreads();
  float* red = reinterpret_cast<float*>(sm);   // 4 x NT x 4 x 32 floats (ConvSmem checks)
  if (kh) {
#pragma unroll
    for (int q = 0; q < NT; ++q)
#pragma unroll
      for (int e = 0; e < 4; ++e) red[((prow * NT + q) * 4 + e) * 32 + lane] = acc[q][e];
  }
  __syncthreads();
  if (kh) return;
#pragma unroll
  for (int q = 0; q < NT; ++q)
#pragma unroll
    for (int e = 0; e < 4; ++e) acc[q][e] += red[((prow * NT + q) * 4 + e) * 32 + lane];
  // epilogue: bias, ReLU, store; with Yp also the 2x2 average pool of the
  // output (the warp holds both rows of a pooling window; the column
  // neighbour is 4 lanes up), summed in the order s00 + s10 + s01 + s11 of the
  // oracle's pool2
  const int gw = w0 + g;
#pragma unroll
  for (int q = 0; q < NT; ++q) {
    const int col = co0 + q * 8 + tg * 2;
    const float b0 = bias ? bias[col] : 0.f, b1 = bias ? bias[col + 1] : 0.f;
    float y[2][2];
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      y[half][0] = acc[q][half * 2] + b0;
      y[half][1] = acc[q][half * 2 + 1] + b1;
      if (relu) {
        y[half][0] = fmaxf(y[half][0], 0.f);
        y[half][1] = fmaxf(y[half][1], 0.f);
      }
      const int gh = h0 + ty0 + half;
      if (gh < H && gw < W)
        *reinterpret_cast<float2*>(&Y[(((long)n * H + gh) * W + gw) * Cout + col]) =
            make_float2(y[half][0], y[half][1]);
    }
    if (Yp) {
      float pv[2];
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        const float s01 = __shfl_down_sync(0xffffffffu, y[0][c], 4);
        const float s11 = __shfl_down_sync(0xffffffffu, y[1][c], 4);
        pv[c] = 0.25f * (((y[0][c] + y[1][c]) + s01) + s11);
      }
      const int ph = (h0 + ty0) >> 1, pw = gw >> 1;
      if (!(g & 1) && h0 + ty0 + 1 < H && gw + 1 < W)
        *reinterpret_cast<float2*>(&Yp[(((long)n * (H / 2) + ph) * (W / 2) + pw) * Cout + col]) =
            make_float2(pv[0], pv[1]);
    }
  }
}

// One 8 x 8 pixel tile t (tiles ordered w fastest, then h, then sample) and
// the BN = NT * 8 output channels from co0.  PDL: dependent launch (wait for
// the previous layer after staging the weights).  Warps 4-7 return before the
// epilogue: nothing after the K halves' hand-over may synchronise the block.
template <int CIN, int NT, bool PDL>
__device__ __forceinline__ void conv_tile(const ConvArgs& cv, int t, int co0,
                                          unsigned char* conv_sm) {
  const float* __restrict__ X = cv.X;
  const int H = cv.H, W = cv.W, Cout = cv.Cout;
  const __nv_bfloat16* __restrict__ WT = cv.WT;
  const float* __restrict__ bias = cv.bias;
  float* __restrict__ Y = cv.Y;
  const int relu = cv.relu;
  float* __restrict__ Yp = cv.Yp;
  const float* __restrict__ Xc = cv.Xc;
  using S = ConvSmem<CIN, NT>;
  constexpr int AS = S::AS, BN = S::BN;
  __nv_bfloat16* As = reinterpret_cast<__nv_bfloat16*>(conv_sm);          // [px][AS] BF16
  __nv_bfloat16* Bs = reinterpret_cast<__nv_bfloat16*>(conv_sm + S::a_bytes);   // [tap][BN][AS]
  const int tid = threadIdx.x;
  const int tilesW = (W + CT - 1) / CT, tilesH = (H + CT - 1) / CT;
  const int tw = t % tilesW;
  t /= tilesW;
  const int th = t % tilesH;
  const int n = t / tilesH;
  const int h0 = th * CT, w0 = tw * CT;
  {  // weights of the 9 taps: 9 * BN rows of CIN BF16, CIN / 8 16-byte pieces each
    constexpr int PR = CIN / 8;
    for (int e = tid; e < 9 * BN * PR; e += CONV_THREADS) {
      const int row = e / PR, q = e - row * PR;
      const int tap = row / BN, r = row - tap * BN;
      cp_async16(Bs + row * AS + q * 8, WT + ((long)tap * Cout + co0 + r) * CIN + q * 8);
    }
    cp_async_commit();
  }
  // the weights do not depend on the previous layer: staged before the wait
  // for the previous layer's output
  if (PDL) pdl_wait();
  {  // the halo tile, rounded once to BF16 (the MMA operands), zeros outside
     // the image.  The FP32 input is formed first exactly as the layer
     // defines it - the features scaled by 1 / their RMS (k_nn_norm's
     // arithmetic), or the decoder's up2(Xc) + X - and rounded as the
     // fragments were before.  Four 8-channel pieces per thread in flight.
    constexpr int C8 = CIN / 8, XB = 4;
    const int Hc = H >> 1, Wc = W >> 1;
    float ir = 1.f, ip = 1.f;
    if (cv.norm) {
      ir = (float)(1.0 / cv.norm->nn_rms_r);
      ip = (float)(1.0 / cv.norm->nn_rms_p);
    }
    for (int e0 = tid; e0 < CT_HALO * C8; e0 += XB * CONV_THREADS) {
      float4 xa[XB], xb[XB], ca[XB], cb[XB];
      bool in[XB];
#pragma unroll
      for (int k = 0; k < XB; ++k) {
        const int e = e0 + k * CONV_THREADS;
        const int px = e / C8, q = e - px * C8;
        const int hy = px / (CT + 2), hx = px - hy * (CT + 2);
        const int gh = h0 - 1 + hy, gw = w0 - 1 + hx;
        in[k] = e < CT_HALO * C8 && gh >= 0 && gh < H && gw >= 0 && gw < W;
        xa[k] = xb[k] = ca[k] = cb[k] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (in[k]) {
          const float4* src =
              reinterpret_cast<const float4*>(X + (((long)n * H + gh) * W + gw) * CIN + q * 8);
          xa[k] = __ldcg(src);
          xb[k] = __ldcg(src + 1);
          if (Xc) {
            const float4* cs = reinterpret_cast<const float4*>(
                Xc + (((long)n * Hc + (gh >> 1)) * Wc + (gw >> 1)) * CIN + q * 8);
            ca[k] = __ldcg(cs);
            cb[k] = __ldcg(cs + 1);
          }
        }
      }
#pragma unroll
      for (int k = 0; k < XB; ++k) {
        const int e = e0 + k * CONV_THREADS;
        if (e >= CT_HALO * C8) break;
        const int px = e / C8, q = e - px * C8;
        float4 a = xa[k], b = xb[k];
        if (cv.norm && q == 0) {
          a.x *= ir;
          a.z *= ip;
        }
        if (Xc && in[k]) {
          a = make_float4(ca[k].x + a.x, ca[k].y + a.y, ca[k].z + a.z, ca[k].w + a.w);
          b = make_float4(cb[k].x + b.x, cb[k].y + b.y, cb[k].z + b.z, cb[k].w + b.w);
        }
        uint4 v;
        v.x = pack_bf16x2(a.x, a.y);
        v.y = pack_bf16x2(a.z, a.w);
        v.z = pack_bf16x2(b.x, b.y);
        v.w = pack_bf16x2(b.z, b.w);
        *reinterpret_cast<uint4*>(As + px * AS + q * 8) = v;
      }
    }
  }
  cp_async_wait<0>();
  __syncthreads();
  conv_core<CIN, NT>(As, Bs, conv_sm, ConvOut{Y, Yp, bias, relu, H, W, Cout, n, h0, w0, co0});
}

template <int CIN, int NT>
__global__ void __launch_bounds__(CONV_THREADS) k_conv3x3(ConvArgs a) {
  extern __shared__ __align__(16) unsigned char conv_sm[];
  conv_tile<CIN, NT, true>(a, blockIdx.x, blockIdx.y * NT * 8, conv_sm);
}

// ---------------------------------------------------------------- layer pairs
// Two 3x3 convolutions at the same resolution in one launch (inference):
// phase A computes the first layer on the 10 x 10 region around the output
// tile - the second layer's halo - from a 12 x 12 input halo, as seven
// 16-row fragments whose rows ldmatrix addresses pixel by pixel (100 of the
// 112 rows are used), and stores it, bias and ReLU applied, rounded to BF16
// (the rounding the second layer's staging applies) and zero outside the
// image (the second layer's 'SAME' padding), in shared memory; phase B is
// conv_core on that intermediate.  The first layer's output never leaves
// the SM, and the pair costs one launch and one staging round.  Used for the
// full-resolution pairs (e0a/e0b, d0a/d0b), whose 256 tiles fill the GPU;
// at 128 x 32 (e1a/e1b: 64 tiles of 64 channels) the fused pair measured
// slower than two launches of 256 lighter blocks, and the deeper pairs keep
// one launch per layer, where splitting the output channels over blocks is
// the parallelism.
template <int CIN, int CMID, int COUT>
struct PairSmem {
  static constexpr int ASI = CIN + 8, ASM = CMID + 8;
  static constexpr int HE = CT + 4, HIN = HE * HE;   // 12 x 12 input halo
  static constexpr size_t in_bytes = (size_t)HIN * ASI * 2;
  static constexpr size_t wa_bytes = (size_t)9 * CMID * ASI * 2;
  static constexpr size_t mid_bytes = (size_t)CT_HALO * ASM * 2;
  static constexpr size_t wb_bytes = (size_t)9 * COUT * ASM * 2;
  static constexpr size_t off_wa = in_bytes, off_mid = off_wa + wa_bytes,
                          off_wb = off_mid + mid_bytes, bytes = off_wb + wb_bytes;
  static_assert(in_bytes % 16 == 0 && wa_bytes % 16 == 0 && mid_bytes % 16 == 0 &&
                    (ASI * 2) % 16 == 0 && (ASM * 2) % 16 == 0,
                "ldmatrix rows and sections 16-byte aligned");
  static_assert((size_t)4 * (COUT / 8) * 4 * 32 * 4 <= off_mid,
                "the K halves' hand-over fits the dead input sections");
};

struct PairArgs {
  const float* X;        // first layer's input, NHWC [H][W][CIN]
  const float* Xc;       // nullable: the input is up2(Xc) + X
  const DevScalars* norm;   // nullable: scale input channels 0 and 2 (the features)
  int H, W;
  const __nv_bfloat16* WA;  // [tap][CMID][CIN]
  const float* biasA;
  int reluA;
  const __nv_bfloat16* WB;  // [tap][COUT][CMID]
  const float* biasB;
  int reluB;
  float* Y;              // second layer's output [H][W][COUT]
  float* Yp;             // nullable: its 2x2 average pool
};

template <int CIN, int CMID, int COUT>
__global__ void __launch_bounds__(CONV_THREADS) k_conv_pair(PairArgs a) {
  extern __shared__ __align__(16) unsigned char pair_sm[];
  using S = PairSmem<CIN, CMID, COUT>;
  constexpr int ASI = S::ASI, ASM = S::ASM, HE = S::HE;
  __nv_bfloat16* In = reinterpret_cast<__nv_bfloat16*>(pair_sm);
  __nv_bfloat16* Wa = reinterpret_cast<__nv_bfloat16*>(pair_sm + S::off_wa);
  __nv_bfloat16* Mid = reinterpret_cast<__nv_bfloat16*>(pair_sm + S::off_mid);
  __nv_bfloat16* Wb = reinterpret_cast<__nv_bfloat16*>(pair_sm + S::off_wb);
  const int H = a.H, W = a.W;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int g = lane >> 2, tg = lane & 3;
  const int tilesW = (W + CT - 1) / CT;
  const int h0 = (blockIdx.x / tilesW) * CT, w0 = (blockIdx.x % tilesW) * CT;
  {  // both layers' weights (all channels), before the wait for the input
    constexpr int PRA = CIN / 8, PRB = CMID / 8;
    for (int e = tid; e < 9 * CMID * PRA; e += CONV_THREADS) {
      const int row = e / PRA, q = e - row * PRA;
      cp_async16(Wa + row * ASI + q * 8, a.WA + (long)row * CIN + q * 8);
    }
    for (int e = tid; e < 9 * COUT * PRB; e += CONV_THREADS) {
      const int row = e / PRB, q = e - row * PRB;
      cp_async16(Wb + row * ASM + q * 8, a.WB + (long)row * CMID + q * 8);
    }
    cp_async_commit();
  }
  pdl_wait();
  {  // the 12 x 12 input halo in BF16 (conv_tile's staging, two cells deep)
    constexpr int C8 = CIN / 8, XB = 4;
    const int Hc = H >> 1, Wc = W >> 1;
    float ir = 1.f, ip = 1.f;
    if (a.norm) {
      ir = (float)(1.0 / a.norm->nn_rms_r);
      ip = (float)(1.0 / a.norm->nn_rms_p);
    }
    for (int e0 = tid; e0 < S::HIN * C8; e0 += XB * CONV_THREADS) {
      float4 xa[XB], xb[XB], ca[XB], cb[XB];
      bool in[XB];
#pragma unroll
      for (int k = 0; k < XB; ++k) {
        const int e = e0 + k * CONV_THREADS;
        const int px = e / C8, q = e - px * C8;
        const int hy = px / HE, hx = px - hy * HE;
        const int gh = h0 - 2 + hy, gw = w0 - 2 + hx;
        in[k] = e < S::HIN * C8 && gh >= 0 && gh < H && gw >= 0 && gw < W;
        xa[k] = xb[k] = ca[k] = cb[k] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (in[k]) {
          const float4* src = reinterpret_cast<const float4*>(a.X + ((long)gh * W + gw) * CIN + q * 8);
          xa[k] = __ldcg(src);
          xb[k] = __ldcg(src + 1);
          if (a.Xc) {
            const float4* cs = reinterpret_cast<const float4*>(
                a.Xc + ((long)(gh >> 1) * Wc + (gw >> 1)) * CIN + q * 8);
            ca[k] = __ldcg(cs);
            cb[k] = __ldcg(cs + 1);
          }
        }
      }
#pragma unroll
      for (int k = 0; k < XB; ++k) {
        const int e = e0 + k * CONV_THREADS;
        if (e >= S::HIN * C8) break;
        const int px = e / C8, q = e - px * C8;
        float4 u = xa[k], w = xb[k];
        if (a.norm && q == 0) {
          u.x *= ir;
          u.z *= ip;
        }
        if (a.Xc && in[k]) {
          u = make_float4(ca[k].x + u.x, ca[k].y + u.y, ca[k].z + u.z, ca[k].w + u.w);
          w = make_float4(cb[k].x + w.x, cb[k].y + w.y, cb[k].z + w.z, cb[k].w + w.w);
        }
        uint4 v;
        v.x = pack_bf16x2(u.x, u.y);
        v.y = pack_bf16x2(u.z, u.w);
        v.z = pack_bf16x2(w.x, w.y);
        v.w = pack_bf16x2(w.z, w.w);
        *reinterpret_cast<uint4*>(In + px * ASI + q * 8) = v;
      }
    }
    (void)Hc;
  }
  cp_async_wait<0>();
  __syncthreads();
  // phase A: warp w < 7 computes rows 16 w .. 16 w + 15 of the 10 x 10
  // intermediate (pixel p = 10 py + px at (h0 - 1 + py, w0 - 1 + px)), all
  // CMID channels, the nine taps in order with even and odd 16-channel steps
  // in separate accumulators
  if (warp < 7) {
    constexpr int NQ = CMID / 8;
    float acc[NQ][4], acc2[NQ][4];
#pragma unroll
    for (int q = 0; q < NQ; ++q)
#pragma unroll
      for (int e = 0; e < 4; ++e) acc[q][e] = acc2[q][e] = 0.f;
    const int lm = lane >> 3, lr = lane & 7;
    int pr = warp * 16 + (lm & 1) * 8 + lr;   // this lane's ldmatrix row (a pixel)
    pr = pr < CT_HALO ? pr : CT_HALO - 1;     // rows 100..111: any valid pixel, discarded
    const int py = pr / (CT + 2), pxx = pr - py * (CT + 2);
    const unsigned in0 = (unsigned)__cvta_generic_to_shared(In);
    const unsigned wa0 = (unsigned)__cvta_generic_to_shared(Wa);
#pragma unroll 1
    for (int tap = 0; tap < 9; ++tap) {
      const int dy = tap / 3, dx = tap % 3;
      const unsigned a_row =
          in0 + (unsigned)((((py + dy) * HE + pxx + dx) * ASI + (lm >> 1) * 8) * 2);
      const unsigned b_row =
          wa0 + (unsigned)(((tap * CMID + (lm >> 1) * 8 + lr) * ASI + (lm & 1) * 8) * 2);
#pragma unroll
      for (int ks = 0; ks < CIN / 16; ++ks) {
        uint32_t af[4];
        ldsm_x4(af, a_row + ks * 32);
#pragma unroll
        for (int qp = 0; qp < NQ / 2; ++qp) {
          uint32_t b[4];
          ldsm_x4(b, b_row + (unsigned)(qp * 16 * ASI * 2) + ks * 32);
          mma_bf16((ks & 1) ? acc2[2 * qp] : acc[2 * qp], af, b);
          mma_bf16((ks & 1) ? acc2[2 * qp + 1] : acc[2 * qp + 1], af, b + 2);
        }
      }
    }
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const int pix = warp * 16 + g + 8 * half;
      if (pix >= CT_HALO) continue;
      const int qy = pix / (CT + 2), qx = pix - qy * (CT + 2);
      const int gh = h0 - 1 + qy, gw = w0 - 1 + qx;
      const bool inside = gh >= 0 && gh < H && gw >= 0 && gw < W;
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        const int col = q * 8 + tg * 2;
        float v0 = acc[q][half * 2] + acc2[q][half * 2] + a.biasA[col];
        float v1 = acc[q][half * 2 + 1] + acc2[q][half * 2 + 1] + a.biasA[col + 1];
        if (a.reluA) {
          v0 = fmaxf(v0, 0.f);
          v1 = fmaxf(v1, 0.f);
        }
        if (!inside) v0 = v1 = 0.f;
        *reinterpret_cast<uint32_t*>(Mid + pix * ASM + col) = pack_bf16x2(v0, v1);
      }
    }
  }
  __syncthreads();
  // phase B: the second layer on the intermediate, all COUT channels
  conv_core<CMID, COUT / 8>(Mid, Wb, pair_sm,
                            ConvOut{a.Y, a.Yp, a.biasB, a.reluB, H, W, COUT, 0, h0, w0, 0});
}

template <int CIN, int CMID, int COUT>
static void pair_launch(const PairArgs& a, cudaStream_t st) {
  const int tiles = ((a.W + CT - 1) / CT) * ((a.H + CT - 1) / CT);
  launch_pdl(true, k_conv_pair<CIN, CMID, COUT>, dim3(tiles), dim3(CONV_THREADS),
             PairSmem<CIN, CMID, COUT>::bytes, st, a);
}

// AEROJAX_NN_PAIRS=0: every layer its own launch (read once)
static bool nn_pairs_enabled() {
  static const bool on = [] {
    const char* e = getenv("AEROJAX_NN_PAIRS");
    return !(e && e[0] == '0');
  }();
  return on;
}
int nn_inference_conv_launches() { return nn_pairs_enabled() ? 10 : 12; }

template <int CIN, int NT>
static void conv_launch(const float* X, int N, int H, int W, int Cout, const __nv_bfloat16* WT,
                        const float* bias, float* Y, int relu, float* Yp, const float* Xc,
                        cudaStream_t st, bool pdl, const DevScalars* norm) {
  using S = ConvSmem<CIN, NT>;
  const int tiles = ((W + CT - 1) / CT) * ((H + CT - 1) / CT) * N;
  dim3 grid(tiles, Cout / S::BN);
  launch_pdl(pdl, k_conv3x3<CIN, NT>, grid, dim3(CONV_THREADS), S::bytes, st,
             ConvArgs{X, N, H, W, Cout, WT, bias, Y, relu, Yp, Xc, norm});
}

template <int CIN, int NT>
static void conv_attr() {
  cudaFuncSetAttribute(k_conv3x3<CIN, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)ConvSmem<CIN, NT>::bytes);
}
// the dynamic shared-memory opt-in of every convolution instance (once, before
// any launch or capture)
static void conv_attrs() {
  static bool done = false;
  if (done) return;
  conv_attr<16, 2>(); conv_attr<16, 4>();
  conv_attr<32, 2>(); conv_attr<32, 4>();
  conv_attr<64, 2>(); conv_attr<64, 4>();
  conv_attr<128, 2>(); conv_attr<128, 4>();
  cudaFuncSetAttribute(k_conv_pair<16, 32, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)PairSmem<16, 32, 32>::bytes);
  cudaFuncSetAttribute(k_conv_pair<32, 32, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)PairSmem<32, 32, 16>::bytes);

  done = true;
}

template <int CIN>
static int conv_cin(const float* X, int N, int H, int W, int Cout, const __nv_bfloat16* WT,
                    const float* bias, float* Y, int relu, float* Yp, const float* Xc,
                    cudaStream_t st, bool pdl, const DevScalars* norm) {
  // 32 output channels per block, or 16 when that leaves fewer blocks than
  // SMs (the small grids of the deep layers are latency-bound: more, lighter
  // blocks load their weights sooner)
  const long tiles = (long)((W + CT - 1) / CT) * ((H + CT - 1) / CT) * N;
  const bool narrow = Cout == 16 || tiles * (Cout / 32) < 152;
  switch (Cout) {
    case 16:
    case 32:
    case 64:
    case 128:
      if (narrow) conv_launch<CIN, 2>(X, N, H, W, Cout, WT, bias, Y, relu, Yp, Xc, st, pdl, norm);
      else conv_launch<CIN, 4>(X, N, H, W, Cout, WT, bias, Y, relu, Yp, Xc, st, pdl, norm);
      break;
    default: return AJ_ERR_PARAM;
  }
  return AJ_OK;
}

// Y = conv(X, WT) (+ bias, ReLU); WT[tap][Cout][Cin] BF16; Yp (nullable,
// H and W even) receives the 2x2 average pool of Y; with Xc (nullable) the
// input is up2(Xc) + X.  pdl: dependent launch (the weights WT must be
// complete before the chain of dependent launches started)
static int conv3x3(const float* X, int N, int H, int W, int Cin, int Cout,
                   const __nv_bfloat16* WT, const float* bias, float* Y, int relu,
                   cudaStream_t st, float* Yp = nullptr, const float* Xc = nullptr,
                   bool pdl = false, const DevScalars* norm = nullptr) {
  switch (Cin) {
    case 16: return conv_cin<16>(X, N, H, W, Cout, WT, bias, Y, relu, Yp, Xc, st, pdl, norm);
    case 32: return conv_cin<32>(X, N, H, W, Cout, WT, bias, Y, relu, Yp, Xc, st, pdl, norm);
    case 64: return conv_cin<64>(X, N, H, W, Cout, WT, bias, Y, relu, Yp, Xc, st, pdl, norm);
    case 128: return conv_cin<128>(X, N, H, W, Cout, WT, bias, Y, relu, Yp, Xc, st, pdl, norm);
    default: return AJ_ERR_PARAM;
  }
}

// ---------------------------------------------------------------- weight gradient
// dW[tap][ci][co] += sum_p Xshift(p)[ci] * dZ[p][co]: GEMM with M = Cin,
// N = Cout, K = pixels.  One block per (tap, pixel chunk); 8 warps share the
// (Cin/16) x (Cout/8) output tiles; the partial sums are added atomically.
constexpr int DW_THREADS = 256, DW_KC = 64, DW_CHUNK = 4096;
constexpr int DW_S = DW_KC + 8;     // bf16 row stride of the staged tiles

__global__ void __launch_bounds__(DW_THREADS) k_conv_dw(const float* __restrict__ X,
                                                        const float* __restrict__ dZ, int N, int H,
                                                        int W, int Cin, int Cout,
                                                        float* __restrict__ dW) {
  __shared__ __align__(16) __nv_bfloat16 As[128 * DW_S];   // [ci][px]
  __shared__ __align__(16) __nv_bfloat16 Bs[128 * DW_S];   // [co][px]
  const int tap = blockIdx.y;
  const int dy = tap / 3 - 1, dx = tap % 3 - 1;
  const long P = (long)N * H * W;
  const long pbeg = (long)blockIdx.x * DW_CHUNK;
  const long pend = pbeg + DW_CHUNK < P ? pbeg + DW_CHUNK : P;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int g = lane >> 2, tg = lane & 3;
  const int MT = Cin / 16, NTt = Cout / 8, ntiles = MT * NTt;
  constexpr int MAXT = 16;          // tiles per warp (128x128 / 8 warps / (16x8))
  float acc[MAXT][4];
#pragma unroll
  for (int q = 0; q < MAXT; ++q) acc[q][0] = acc[q][1] = acc[q][2] = acc[q][3] = 0.f;
  for (long pc = pbeg; pc < pend; pc += DW_KC) {
    // stage X shifted (transposed to [ci][px]) and dZ (transposed to [co][px])
    for (int e = tid; e < DW_KC * Cin; e += DW_THREADS) {
      const int px = e / Cin, ci = e - px * Cin;
      const long p = pc + px;
      float v = 0.f;
      if (p < pend) {
        const int n = (int)(p / ((long)H * W));
        const int rem = (int)(p - (long)n * H * W);
        const int h = rem / W + dy, w = rem % W + dx;
        if (h >= 0 && h < H && w >= 0 && w < W) v = X[(((long)n * H + h) * W + w) * Cin + ci];
      }
      As[ci * DW_S + px] = __float2bfloat16_rn(v);
    }
    for (int e = tid; e < DW_KC * Cout; e += DW_THREADS) {
      const int px = e / Cout, co = e - px * Cout;
      const long p = pc + px;
      Bs[co * DW_S + px] = __float2bfloat16_rn(p < pend ? dZ[p * Cout + co] : 0.f);
    }
    __syncthreads();
#pragma unroll
    for (int ks = 0; ks < DW_KC; ks += 16) {
#pragma unroll
      for (int q = 0; q < MAXT; ++q) {
        const int tile = warp + q * 8;
        if (tile >= ntiles) break;
        const int mt = tile / NTt, nt = tile - mt * NTt;
        const int r = mt * 16 + g;
        uint32_t a[4], b[2];
        a[0] = *reinterpret_cast<const uint32_t*>(&As[r * DW_S + ks + tg * 2]);
        a[1] = *reinterpret_cast<const uint32_t*>(&As[(r + 8) * DW_S + ks + tg * 2]);
        a[2] = *reinterpret_cast<const uint32_t*>(&As[r * DW_S + ks + tg * 2 + 8]);
        a[3] = *reinterpret_cast<const uint32_t*>(&As[(r + 8) * DW_S + ks + tg * 2 + 8]);
        const int n = nt * 8 + g;
        b[0] = *reinterpret_cast<const uint32_t*>(&Bs[n * DW_S + ks + tg * 2]);
        b[1] = *reinterpret_cast<const uint32_t*>(&Bs[n * DW_S + ks + tg * 2 + 8]);
        mma_bf16(acc[q], a, b);
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < MAXT; ++q) {
    const int tile = warp + q * 8;
    if (tile >= ntiles) break;
    const int mt = tile / NTt, nt = tile - mt * NTt;
    const int col = nt * 8 + tg * 2;
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const int ci = mt * 16 + g + half * 8;
      float* dst = dW + ((long)tap * Cin + ci) * Cout + col;
      atomicAdd(dst, acc[q][half * 2]);
      atomicAdd(dst + 1, acc[q][half * 2 + 1]);
    }
  }
}

// db[co] += sum_p dZ[p][co]
__global__ void k_bias_grad(const float* __restrict__ dZ, long P, int C, float* __restrict__ db) {
  const int co = threadIdx.x % C;
  const int lanes = blockDim.x / C;
  const int li = threadIdx.x / C;
  if (li >= lanes) return;
  float s = 0.f;
  for (long p = (long)blockIdx.x * lanes + li; p < P; p += (long)gridDim.x * lanes) s += dZ[p * C + co];
  atomicAdd(&db[co], s);
}

// ---------------------------------------------------------------- element-wise
// dX (fine, accumulated) += pool2 adjoint of dY (coarse)
__global__ void k_pool2_bwd(const float* __restrict__ dY, float* __restrict__ dX, int N, int H,
                            int W, int C) {   // H, W of dY
  long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const long T = (long)N * 2 * H * 2 * W * C;
  if (e >= T) return;
  const int c = (int)(e % C);
  long q = e / C;
  const int w = (int)(q % (2 * W));
  q /= 2 * W;
  const int h = (int)(q % (2 * H));
  const int n = (int)(q / (2 * H));
  dX[e] += 0.25f * dY[(((long)n * H + h / 2) * W + w / 2) * C + c];
}

// Y (fine) = up2(X coarse) + S (fine)
__global__ void k_up2_add(const float* __restrict__ X, const float* __restrict__ S,
                          float* __restrict__ Y, int N, int H, int W, int C) {   // fine H, W
  long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const long T = (long)N * H * W * C;
  if (e >= T) return;
  const int c = (int)(e % C);
  long q = e / C;
  const int w = (int)(q % W);
  q /= W;
  const int h = (int)(q % H);
  const int n = (int)(q / H);
  Y[e] = X[(((long)n * (H / 2) + h / 2) * (W / 2) + w / 2) * C + c] + S[e];
}

// dX (coarse) = adjoint of nearest up2 applied to dY (fine)
__global__ void k_up2_bwd(const float* __restrict__ dY, float* __restrict__ dX, int N, int H,
                          int W, int C) {   // coarse H, W
  long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const long T = (long)N * H * W * C;
  if (e >= T) return;
  const int c = (int)(e % C);
  long q = e / C;
  const int w = (int)(q % W);
  q /= W;
  const int h = (int)(q % H);
  const int n = (int)(q / H);
  const int W2 = 2 * W;
  const long b = (((long)n * 2 * H + 2 * h) * W2 + 2 * w) * C + c;
  dX[e] = dY[b] + dY[b + (long)W2 * C] + dY[b + C] + dY[b + (long)W2 * C + C];
}

// dZ = dOut * (Y > 0)   (ReLU adjoint)
__global__ void k_relu_gate(const float* __restrict__ dOut, const float* __restrict__ Y,
                            float* __restrict__ dZ, long T) {
  long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (e < T) dZ[e] = Y[e] > 0.f ? dOut[e] : 0.f;
}

// loss = mean over pixels of (y[.,0] - target)^2; dy = its gradient
__global__ void k_mse(const float* __restrict__ y, const float* __restrict__ target,
                      float* __restrict__ dy, long P, double* loss) {
  float s = 0.f;
  const float inv = 1.f / (float)P;
  for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < P; p += (long)gridDim.x * blockDim.x) {
    const float d = y[p * 16] - target[p];
    s = fmaf(d, d, s);
    dy[p * 16] = 2.f * d * inv;
#pragma unroll
    for (int c = 1; c < 16; ++c) dy[p * 16 + c] = 0.f;
  }
  block_sum_atomic((double)s * (double)inv, loss);
}

// Adam with element-wise clipping of the gradient to [-clip, clip]
__global__ void k_adam(float* __restrict__ w, const float* __restrict__ gr, float* __restrict__ m,
                       float* __restrict__ v, long n, float lr, float b1, float b2, float eps,
                       float clip, float c1, float c2) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  float g = fminf(fmaxf(gr[i], -clip), clip);
  float mi = b1 * m[i] + (1.f - b1) * g;
  float vi = b2 * v[i] + (1.f - b2) * g * g;
  m[i] = mi;
  v[i] = vi;
  w[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
}

struct PackTab {
  int nl;
  long woff[NL], poff[NL];
  int cin[NL], cout[NL];
};

// FP32 master weights -> BF16 WfT[tap][co][ci] (forward) and
// WbT[8-tap][ci][co] (the adjoint: output channel ci, input channel co)
__global__ void k_pack(const float* __restrict__ master, __nv_bfloat16* __restrict__ packed,
                       PackTab tab) {
  const int l = blockIdx.y;
  const int cin = tab.cin[l], cout = tab.cout[l];
  const long nw = 9L * cin * cout;
  const float* W = master + tab.woff[l];
  __nv_bfloat16* Wf = packed + tab.poff[l];
  __nv_bfloat16* Wb = Wf + nw;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < nw; e += (long)gridDim.x * blockDim.x) {
    const int co = (int)(e % cout);
    const long q = e / cout;
    const int ci = (int)(q % cin);
    const int tap = (int)(q / cin);
    const __nv_bfloat16 b = __float2bfloat16_rn(W[e]);
    Wf[((long)tap * cout + co) * cin + ci] = b;
    Wb[((long)(8 - tap) * cin + ci) * cout + co] = b;
  }
}

static PackTab pack_tab() {
  PackTab t;
  t.nl = NL;
  for (int l = 0; l < NL; ++l) {
    t.woff[l] = (long)w_off(l);
    t.poff[l] = (long)pk_off(l);
    t.cin[l] = kLayers[l].cin;
    t.cout[l] = kLayers[l].cout;
  }
  return t;
}

// ---------------------------------------------------------------- activations
// Every tensor the backward pass needs, for batch n at the network grid h x w.
struct NnActs {
  float *x, *a0, *s0, *p0, *a1, *s1, *p1, *a2, *s2, *p2, *a3, *bt;
  float *u2, *o2, *u1, *o1, *u0, *o0, *y;
  // backward: skip-connection gradients and two scratch buffers per resolution
  float *ds0, *ds1, *ds2, *sa0, *sa1, *sb1, *sa2, *sb2, *sa3, *sb3;
  size_t total;
};

static NnActs act_layout(int n, int h, int w, void* base) {
  NnActs A;
  size_t off = 0;
  char* b = static_cast<char*>(base);
  auto take = [&](long elems) {
    float* p = reinterpret_cast<float*>(b ? b + off : nullptr);
    off += ((size_t)elems * 4 + 255) & ~(size_t)255;
    return p;
  };
  const long P0 = (long)n * h * w, P1 = P0 / 4, P2 = P0 / 16, P3 = P0 / 64;
  A.x = take(P0 * 16);
  A.a0 = take(P0 * 32);
  A.s0 = take(P0 * 32);
  A.p0 = take(P1 * 32);
  A.a1 = take(P1 * 64);
  A.s1 = take(P1 * 64);
  A.p1 = take(P2 * 64);
  A.a2 = take(P2 * 128);
  A.s2 = take(P2 * 128);
  A.p2 = take(P3 * 128);
  A.a3 = take(P3 * 128);
  A.bt = take(P3 * 128);
  A.u2 = take(P2 * 128);
  A.o2 = take(P2 * 64);
  A.u1 = take(P1 * 64);
  A.o1 = take(P1 * 32);
  A.u0 = take(P0 * 32);
  A.o0 = take(P0 * 32);
  A.y = take(P0 * 16);
  A.ds0 = take(P0 * 32);
  A.sa0 = take(P0 * 32);
  A.ds1 = take(P1 * 64);
  A.sa1 = take(P1 * 64);
  A.sb1 = take(P1 * 32);
  A.ds2 = take(P2 * 128);
  A.sa2 = take(P2 * 128);
  A.sb2 = take(P2 * 64);
  A.sa3 = take(P3 * 128);
  A.sb3 = take(P3 * 128);
  A.total = off;
  return A;
}

struct NnW {
  const __nv_bfloat16* packed;
  const float* master;
  const __nv_bfloat16* wf(int l) const { return packed + pk_off(l); }
  const __nv_bfloat16* wb(int l) const {
    return packed + pk_off(l) + 9 * (size_t)kLayers[l].cin * kLayers[l].cout;
  }
  const float* bias(int l) const { return master + b_off(l); }
};

static inline unsigned ew_blocks(long T) { return cdiv(T, 256); }

// The forward pass.  keep: materialise the decoder inputs u = up2(o) + s
// (the backward pass needs them); else the decoder convolutions add the
// up-sampled coarse input while staging their halo (inference).
int nn_forward(int n, int h, int w, const NnW& W, const NnActs& A, cudaStream_t st,
               bool keep = true, const DevScalars* norm = nullptr) {
  const int H0 = h, W0 = w, H1 = h / 2, W1 = w / 2, H2 = h / 4, W2 = w / 4, H3 = h / 8, W3 = w / 8;
  // inference launches the convolutions as one chain of dependent launches
  auto conv = [&](int l, const float* in, float* out, int H, int Wd, float* pooled = nullptr,
                  const float* coarse = nullptr) {
    return conv3x3(in, n, H, Wd, kLayers[l].cin, kLayers[l].cout, W.wf(l), W.bias(l), out,
                   kLayers[l].relu, st, pooled, coarse, !keep, l == E0A ? norm : nullptr);
  };
  int rc = AJ_OK;
  // inference on one sample: the full-resolution layer pairs in one launch each
  const bool pairs = !keep && n == 1 && nn_pairs_enabled();
  if (pairs) {
    pair_launch<16, 32, 32>(PairArgs{A.x, nullptr, norm, H0, W0, W.wf(E0A), W.bias(E0A),
                                     kLayers[E0A].relu, W.wf(E0B), W.bias(E0B),
                                     kLayers[E0B].relu, A.s0, A.p0}, st);
  } else {
    rc |= conv(E0A, A.x, A.a0, H0, W0);
    rc |= conv(E0B, A.a0, A.s0, H0, W0, A.p0);   // s0 and its pool p0
  }
  rc |= conv(E1A, A.p0, A.a1, H1, W1);
  rc |= conv(E1B, A.a1, A.s1, H1, W1, A.p1);
  rc |= conv(E2A, A.p1, A.a2, H2, W2);
  rc |= conv(E2B, A.a2, A.s2, H2, W2, A.p2);
  rc |= conv(E3A, A.p2, A.a3, H3, W3);
  rc |= conv(E3B, A.a3, A.bt, H3, W3);
  if (keep) {
    k_up2_add<<<ew_blocks((long)n * H2 * W2 * 128), 256, 0, st>>>(A.bt, A.s2, A.u2, n, H2, W2, 128);
    rc |= conv(D2, A.u2, A.o2, H2, W2);
    k_up2_add<<<ew_blocks((long)n * H1 * W1 * 64), 256, 0, st>>>(A.o2, A.s1, A.u1, n, H1, W1, 64);
    rc |= conv(D1, A.u1, A.o1, H1, W1);
    k_up2_add<<<ew_blocks((long)n * H0 * W0 * 32), 256, 0, st>>>(A.o1, A.s0, A.u0, n, H0, W0, 32);
    rc |= conv(D0A, A.u0, A.o0, H0, W0);
  } else {
    rc |= conv(D2, A.s2, A.o2, H2, W2, nullptr, A.bt);
    rc |= conv(D1, A.s1, A.o1, H1, W1, nullptr, A.o2);
    if (pairs)
      pair_launch<32, 32, 16>(PairArgs{A.s0, A.o1, nullptr, H0, W0, W.wf(D0A), W.bias(D0A),
                                       kLayers[D0A].relu, W.wf(D0B), W.bias(D0B),
                                       kLayers[D0B].relu, A.y, nullptr}, st);
    else
      rc |= conv(D0A, A.s0, A.o0, H0, W0, nullptr, A.o1);
  }
  if (!pairs) rc |= conv(D0B, A.o0, A.y, H0, W0);
  if (rc != AJ_OK) return AJ_ERR_PARAM;
  return cudaGetLastError() == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
}

// gradient of one conv layer: dz = dout (* ReLU gate), dW, db, and (if dx) the
// input gradient
static void layer_bwd(int l, int n, int H, int Wd, const float* in, const float* out,
                      const float* dout, float* dz, float* dx, const NnW& W, float* grad,
                      cudaStream_t st) {
  const int cin = kLayers[l].cin, cout = kLayers[l].cout;
  const long P = (long)n * H * Wd;
  const float* g = dout;
  if (kLayers[l].relu) {
    k_relu_gate<<<ew_blocks(P * cout), 256, 0, st>>>(dout, out, dz, P * cout);
    g = dz;
  }
  dim3 gdw(cdiv(P, DW_CHUNK), 9);
  k_conv_dw<<<gdw, DW_THREADS, 0, st>>>(in, g, n, H, Wd, cin, cout, grad + w_off(l));
  const int lanes = 256 / cout;
  unsigned nb = cdiv(P, (long)lanes * 64);
  if (nb > 512) nb = 512;
  k_bias_grad<<<nb, lanes * cout, 0, st>>>(g, P, cout, grad + b_off(l));
  if (dx) conv3x3(g, n, H, Wd, cout, cin, W.wb(l), nullptr, dx, 0, st);
}

int nn_backward(int n, int h, int w, const float* dy, const NnW& W, const NnActs& A, float* grad,
                cudaStream_t st) {
  const int H0 = h, W0 = w, H1 = h / 2, W1 = w / 2, H2 = h / 4, W2 = w / 4, H3 = h / 8, W3 = w / 8;
  const long P0 = (long)n * H0 * W0, P1 = P0 / 4, P2 = P0 / 16, P3 = P0 / 64;
  if (cudaMemsetAsync(grad, 0, n_params() * 4, st) != cudaSuccess) return AJ_ERR_CUDA;
  // Each layer_bwd gates its incoming gradient in place and writes the input
  // gradient to a different buffer.  Decoder first: y = d0b(o0),
  // o0 = d0a(u0), u0 = up(o1) + s0, ...
  layer_bwd(D0B, n, H0, W0, A.o0, A.y, dy, nullptr, A.sa0, W, grad, st);        // sa0 = d o0
  layer_bwd(D0A, n, H0, W0, A.u0, A.o0, A.sa0, A.sa0, A.ds0, W, grad, st);      // ds0 = d u0
  k_up2_bwd<<<ew_blocks(P1 * 32), 256, 0, st>>>(A.ds0, A.sa1, n, H1, W1, 32);   // sa1 = d o1
  layer_bwd(D1, n, H1, W1, A.u1, A.o1, A.sa1, A.sa1, A.ds1, W, grad, st);       // ds1 = d u1
  k_up2_bwd<<<ew_blocks(P2 * 64), 256, 0, st>>>(A.ds1, A.sa2, n, H2, W2, 64);   // sa2 = d o2
  layer_bwd(D2, n, H2, W2, A.u2, A.o2, A.sa2, A.sa2, A.ds2, W, grad, st);       // ds2 = d u2
  k_up2_bwd<<<ew_blocks(P3 * 128), 256, 0, st>>>(A.ds2, A.sa3, n, H3, W3, 128); // sa3 = d bt
  // encoder: the skip gradients ds* accumulate the pooled paths
  layer_bwd(E3B, n, H3, W3, A.a3, A.bt, A.sa3, A.sa3, A.sb3, W, grad, st);      // sb3 = d a3
  layer_bwd(E3A, n, H3, W3, A.p2, A.a3, A.sb3, A.sb3, A.sa3, W, grad, st);      // sa3 = d p2
  k_pool2_bwd<<<ew_blocks(P2 * 128), 256, 0, st>>>(A.sa3, A.ds2, n, H3, W3, 128);   // ds2 = d s2
  layer_bwd(E2B, n, H2, W2, A.a2, A.s2, A.ds2, A.ds2, A.sa2, W, grad, st);      // sa2 = d a2
  layer_bwd(E2A, n, H2, W2, A.p1, A.a2, A.sa2, A.sa2, A.sb2, W, grad, st);      // sb2 = d p1
  k_pool2_bwd<<<ew_blocks(P1 * 64), 256, 0, st>>>(A.sb2, A.ds1, n, H2, W2, 64);     // ds1 = d s1
  layer_bwd(E1B, n, H1, W1, A.a1, A.s1, A.ds1, A.ds1, A.sa1, W, grad, st);      // sa1 = d a1
  layer_bwd(E1A, n, H1, W1, A.p0, A.a1, A.sa1, A.sa1, A.sb1, W, grad, st);      // sb1 = d p0
  k_pool2_bwd<<<ew_blocks(P0 * 32), 256, 0, st>>>(A.sb1, A.ds0, n, H1, W1, 32);     // ds0 = d s0
  layer_bwd(E0B, n, H0, W0, A.a0, A.s0, A.ds0, A.ds0, A.sa0, W, grad, st);      // sa0 = d a0
  layer_bwd(E0A, n, H0, W0, A.x, A.a0, A.sa0, A.sa0, nullptr, W, grad, st);
  return cudaGetLastError() == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
}

static bool nn_shape_ok(int n, int h, int w) { return n >= 1 && h >= 8 && w >= 8 && h % 8 == 0 && w % 8 == 0; }

// ---------------------------------------------------------------- warm start
// Network inputs on the grid F times coarser than the pressure grid:
//   channel 0: F x F average of the previous pressure's residual b - A p_prev
//              (the reference operator: edge ghosts, outlet row pinned)
//   channel 1: F x F average of the mask
//   channel 2: F x F average of p_prev
// channels 3..15 are zero.  Also the FP64 sums of channel 0^2 and 2^2.
// one thread per fine cell: the F x F window sums reduce across F lanes with
// shuffles and across F rows through shared memory (F in {2, 4, 8}; a
// 32 x 8 block holds whole windows).  With rs.us set (a MAC step), the
// kernel forms the right-hand side b of its cell itself from the predictor's
// u*, v* (k_rhs's arithmetic) and stores it for the solve.
struct RhsSrc {
  const float* us = nullptr;   // null: read b
  const float* vs = nullptr;
  float idx = 0.f, idy = 0.f;
  int outlet = 0;
  const DevScalars* sc = nullptr;
  float* b_out = nullptr;
};
__global__ void __launch_bounds__(256) k_nn_feat(const float* __restrict__ b,
                                                 const float* __restrict__ mask,
                                                 const float* __restrict__ pp, int nx, int ny,
                                                 int F, float ax, float ay, float* __restrict__ x,
                                                 RhsSrc rs) {
  pdl_wait();
  __shared__ float red[3][8][32];
  const int lane = threadIdx.x, row = threadIdx.y;
  const int j = blockIdx.x * 32 + lane, i = blockIdx.y * 8 + row;
  float vr = 0.f, vm = 0.f, vp = 0.f;
  if (i < nx && j < ny) {
    const long k = (long)i * ny + j;
    const float c = pp[k];
    float bk;
    if (rs.us) {
      bk = rhs_mac_cell(rs.us, rs.vs, mask, i, j, nx, ny, rs.idx, rs.idy, rs.sc->dt, rs.outlet);
      rs.b_out[k] = bk;
    } else {
      bk = b[k];
    }
    if (i != nx - 1) {
      const float xp = pp[k + ny];
      const float xm = i > 0 ? pp[k - ny] : c;
      const float yp = j + 1 < ny ? pp[k + 1] : c;
      const float ym = j > 0 ? pp[k - 1] : c;
      vr = bk - (ax * ((xp - c) + (xm - c)) + ay * ((yp - c) + (ym - c)));
    }
    vm = mask[k];
    vp = c;
  }
  for (int o = 1; o < F; o <<= 1) {
    vr += __shfl_xor_sync(0xffffffffu, vr, o);
    vm += __shfl_xor_sync(0xffffffffu, vm, o);
    vp += __shfl_xor_sync(0xffffffffu, vp, o);
  }
  red[0][row][lane] = vr;
  red[1][row][lane] = vm;
  red[2][row][lane] = vp;
  __syncthreads();
  if ((row % F) == 0 && (lane % F) == 0 && i < nx && j < ny) {
    float ar = 0.f, am = 0.f, ap = 0.f;
    for (int q = 0; q < F; ++q) {
      ar += red[0][row + q][lane];
      am += red[1][row + q][lane];
      ap += red[2][row + q][lane];
    }
    const float inv = 1.f / (float)(F * F);
    ar *= inv;
    am *= inv;
    ap *= inv;
    const int w = ny / F;
    float* o = x + ((long)(i / F) * w + j / F) * 16;
    o[0] = ar;
    o[1] = am;
    o[2] = ap;
#pragma unroll
    for (int c = 3; c < 16; ++c) o[c] = 0.f;
  }
}

// per-sample scales: RMS of channels 0 and 2 over the network grid and the
// output scale rms_r * lmin^2 / 10 (a correction solving A dp = r has that
// magnitude).  Each block files its FP64 partial sums in part[2 b], part[2 b
// + 1]; the last block to finish adds them in block order, so the scales -
// and the correction - are bit-reproducible.
constexpr int NN_SCALE_BLOCKS = 32;
static_assert(2 * NN_SCALE_BLOCKS <= kPartials, "the partial sums live in the workspace's part");
__global__ void __launch_bounds__(512) k_nn_scale(const float* __restrict__ x, long cells,
                                                  DevScalars* sc, double lmin2, double* part) {
  pdl_wait();
  float sr = 0.f, sp = 0.f;
  const long stride = (long)gridDim.x * blockDim.x;
#pragma unroll 4
  for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < cells; c += stride) {
    const float r = x[c * 16], q = x[c * 16 + 2];
    sr = fmaf(r, r, sr);
    sp = fmaf(q, q, sp);
  }
  const double br = block_sum((double)sr);
  const double bp = block_sum((double)sp);
  __shared__ int am_last;
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = br;
    part[2 * blockIdx.x + 1] = bp;
    __threadfence();
    am_last = atomicAdd(&sc->red_count, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!am_last) return;
  // the last block: every thread loads its partials at once (one thread
  // walking them waited on one L2 round trip per partial), then a fixed-order
  // block sum
  __threadfence();
  double lr = 0.0, lp = 0.0;
  for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
    lr += __ldcg(part + 2 * b);
    lp += __ldcg(part + 2 * b + 1);
  }
  const double tr = block_sum(lr);
  const double tp = block_sum(lp);
  if (threadIdx.x == 0) {
    const double rr = sqrt(tr / (double)cells), rp = sqrt(tp / (double)cells);
    const double rrc = rr > 1e-30 ? rr : 1e-30, rpc = rp > 1e-30 ? rp : 1e-30;
    sc->nn_rms_r = rrc;
    sc->nn_rms_p = rpc;
    sc->nn_out_scale = rrc * lmin2 / 10.0;
    sc->red_count = 0u;
  }
}

// normalise channels 0 and 2 in place; optionally copy the 3 features out
__global__ void k_nn_norm(float* __restrict__ x, float* __restrict__ x3, long cells,
                          const DevScalars* sc) {
  pdl_wait();
  const long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (c >= cells) return;
  const float ir = (float)(1.0 / sc->nn_rms_r), ip = (float)(1.0 / sc->nn_rms_p);
  float* o = x + c * 16;
  o[0] *= ir;
  o[2] *= ip;
  if (x3) {
    x3[c * 3] = o[0];
    x3[c * 3 + 1] = o[1];
    x3[c * 3 + 2] = o[2];
  }
}

// training target: F x F average of (p_true - p_prev) / out_scale
__global__ void k_nn_target(const float* __restrict__ pt, const float* __restrict__ pp, int nx,
                            int ny, int F, float* __restrict__ target, const DevScalars* sc) {
  const int J = blockIdx.x * blockDim.x + threadIdx.x;
  const int I = blockIdx.y * blockDim.y + threadIdx.y;
  const int h = nx / F, w = ny / F;
  if (I >= h || J >= w) return;
  float a = 0.f;
  for (int di = 0; di < F; ++di)
    for (int dj = 0; dj < F; ++dj) {
      const long k = (long)(I * F + di) * ny + J * F + dj;
      a += pt[k] - pp[k];
    }
  target[(long)I * w + J] = (float)((double)(a / (float)(F * F)) / sc->nn_out_scale);
}

// the correction at fine cell (i, j): bilinear prolongation of the network
// output (channel 0 of 16 on the grid F times coarser) times out_scale
__device__ __forceinline__ float nn_corr_at(const float* __restrict__ y, int nx, int ny, int F,
                                            double out_scale, int i, int j) {
  const int h = nx / F, w = ny / F;
  const float xi = (i + 0.5f) / F - 0.5f, xj = (j + 0.5f) / F - 0.5f;
  int i0 = (int)floorf(xi), j0 = (int)floorf(xj);
  const float ti = xi - i0, tj = xj - j0;
  const int i1 = min(max(i0 + 1, 0), h - 1), j1 = min(max(j0 + 1, 0), w - 1);
  i0 = min(max(i0, 0), h - 1);
  j0 = min(max(j0, 0), w - 1);
  const float v00 = y[((long)i0 * w + j0) * 16], v01 = y[((long)i0 * w + j1) * 16];
  const float v10 = y[((long)i1 * w + j0) * 16], v11 = y[((long)i1 * w + j1) * 16];
  const float v = (1.f - ti) * ((1.f - tj) * v00 + tj * v01) + ti * ((1.f - tj) * v10 + tj * v11);
  return (float)(v * out_scale);
}

// state += the correction, added to the double-FP32 state (hi: N floats, lo:
// N floats) with Knuth's TwoSum; the outlet row stays pinned at 0
__global__ void k_nn_apply(const float* __restrict__ y, int nx, int ny, int F,
                           float* __restrict__ state, const DevScalars* sc) {
  pdl_wait();
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx - 1 || j >= ny) return;
  const long N = (long)nx * ny;
  const long k = (long)i * ny + j;
  const float c = nn_corr_at(y, nx, ny, F, sc->nn_out_scale, i, j);
  const float hi = state[k], lo = state[N + k];
  const float s = hi + c, bb = s - hi;
  const float e = (hi - (s - bb)) + (c - bb) + lo;
  const float s2 = s + e;
  state[k] = s2;
  state[N + k] = e - (s2 - s);
}

// p0 = p_prev + the correction in FP32 (aj_nn_warmstart); the outlet row is
// 0, the value every solve pins there
__global__ void k_nn_apply_guess(const float* __restrict__ y, int nx, int ny, int F,
                                 const float* __restrict__ pp, float* __restrict__ p0,
                                 const DevScalars* sc) {
  pdl_wait();
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx || j >= ny) return;
  const long k = (long)i * ny + j;
  p0[k] = i == nx - 1 ? 0.f : pp[k] + nn_corr_at(y, nx, ny, F, sc->nn_out_scale, i, j);
}

// [n][h][w][3] -> [n][h][w][16] (zeros beyond the features)
__global__ void k_nn_expand(const float* __restrict__ x3, float* __restrict__ x16, long cells) {
  const long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (e >= cells * 16) return;
  const long c = e / 16;
  const int ch = (int)(e - c * 16);
  x16[e] = ch < 3 ? x3[c * 3 + ch] : 0.f;
}

// features (+ optional dataset copy and target) for one step's pressure solve
int nn_features(const AjStepParams& p, void* ws, double* part, const float* b, const float* mask,
                const float* pp, const float* pt, float* x16, float* x3, float* target,
                cudaStream_t st, bool pdl, bool normalise, const float* us = nullptr,
                const float* vs = nullptr) {
  const int F = p.nn_factor, h = p.nx / F, w = p.ny / F;
  DevScalars* sc = at<DevScalars>(ws, 0);
  dim3 blk(32, 8), grd(cdiv(w, 32), cdiv(h, 8));
  RhsSrc rs;
  if (us) {   // b formed here (k_rhs's launch arguments for a MAC grid)
    rs.us = us;
    rs.vs = vs;
    rs.idx = (float)(1.0 / p.dx);
    rs.idy = (float)(1.0 / p.dy);
    rs.outlet = p.flow_type == AJ_FLOW_VON_KARMAN;
    rs.sc = sc;
    rs.b_out = const_cast<float*>(b);
  }
  launch_pdl(pdl, k_nn_feat, dim3(cdiv(p.ny, 32), cdiv(p.nx, 8)), blk, 0, st, b, mask, pp, p.nx,
             p.ny, F, (float)(1.0 / (p.dx * p.dx)), (float)(1.0 / (p.dy * p.dy)), x16, rs);
  const double lx = p.nx * p.dx, ly = p.ny * p.dy, lmin = lx < ly ? lx : ly;
  launch_pdl(pdl, k_nn_scale, dim3(NN_SCALE_BLOCKS), dim3(512), 0, st, x16, (long)h * w, sc,
             lmin * lmin, part);
  if (normalise)
    launch_pdl(pdl, k_nn_norm, dim3(cdiv((long)h * w, 256)), dim3(256), 0, st, x16, x3,
               (long)h * w, (const DevScalars*)sc);
  if (pt && target) k_nn_target<<<grd, blk, 0, st>>>(pt, pp, p.nx, p.ny, F, target, sc);
  return cudaGetLastError() == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
}

// the learned warm start inside a converging solve: features of the initial
// state, the network, the correction added to the state
int nn_correct_state(const AjStepParams& p, const Layout& L, void* ws, const float* b,
                     const NnWarm& nn, float* state, cudaStream_t st) {
  conv_attrs();
  const int F = p.nn_factor, h = p.nx / F, w = p.ny / F;
  if (F <= 0 || !L.nn_act) return AJ_ERR_PARAM;
  NnActs A = act_layout(1, h, w, at<char>(ws, L.nn_act));
  // features, network and correction: one chain of dependent launches (the
  // packed weights were written before the step began)
  // (the first convolution normalises the features as it stages them)
  int rc = nn_features(p, ws, at<double>(ws, L.part), b, nn.mask, state, nullptr, A.x, nullptr,
                       nullptr, st, true, false, nn.us, nn.vs);
  if (rc != AJ_OK) return rc;
  NnW W{reinterpret_cast<const __nv_bfloat16*>(nn.packed), nn.master};
  rc = nn_forward(1, h, w, W, A, st, false, at<DevScalars>(ws, 0));
  if (rc != AJ_OK) return rc;
  dim3 blk(32, 8), grd(cdiv(p.ny, 32), cdiv(p.nx, 8));
  launch_pdl(true, k_nn_apply, grd, blk, 0, st, (const float*)A.y, p.nx, p.ny, F, state,
             (const DevScalars*)at<DevScalars>(ws, 0));
  return cudaGetLastError() == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
}

size_t nn_step_act_bytes(const AjStepParams& p) {
  if (p.nn_factor <= 0) return 0;
  return act_layout(1, p.nx / p.nn_factor, p.ny / p.nn_factor, nullptr).total;
}

bool nn_step_shape_ok(const AjStepParams& p) {
  const int F = p.nn_factor;
  if (F <= 0) return true;
  if (F != 2 && F != 4 && F != 8) return false;   // whole windows in a 32 x 8 block
  if (p.nx % F || p.ny % F) return false;
  return nn_shape_ok(1, p.nx / F, p.ny / F);
}

}  // namespace aj

using namespace aj;

extern "C" {

size_t aj_nn_param_count(void) { return n_params(); }
size_t aj_nn_packed_count(void) { return n_packed(); }

size_t aj_nn_act_bytes(int32_t n, int32_t h, int32_t w) {
  if (!nn_shape_ok(n, h, w)) return 0;
  return act_layout(n, h, w, nullptr).total;
}

// the network input [n][h][w][16] inside the activation buffer
float* aj_nn_input(int32_t n, int32_t h, int32_t w, void* act) {
  if (!nn_shape_ok(n, h, w) || !act) return nullptr;
  return act_layout(n, h, w, act).x;
}

int32_t aj_nn_pack(const float* master, uint16_t* packed, void* stream) {
  if (!master || !packed) return AJ_ERR_PARAM;
  conv_attrs();
  dim3 grid(64, NL);
  k_pack<<<grid, 256, 0, (cudaStream_t)stream>>>(master, reinterpret_cast<__nv_bfloat16*>(packed),
                                                   pack_tab());
  return cudaGetLastError() == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
}

int32_t aj_nn_forward(int32_t n, int32_t h, int32_t w, const uint16_t* packed, const float* master,
                      void* act, size_t act_bytes, float* y_out, void* stream) {
  if (!nn_shape_ok(n, h, w) || !packed || !master || !act) return AJ_ERR_PARAM;
  conv_attrs();
  NnActs A = act_layout(n, h, w, act);
  if (act_bytes < A.total) return AJ_ERR_WORKSPACE;
  NnW W{reinterpret_cast<const __nv_bfloat16*>(packed), master};
  cudaStream_t st = (cudaStream_t)stream;
  int rc = nn_forward(n, h, w, W, A, st);
  if (rc != AJ_OK) return rc;
  if (y_out && cudaMemcpyAsync(y_out, A.y, (size_t)n * h * w * 16 * 4, cudaMemcpyDeviceToDevice,
                               st) != cudaSuccess)
    return AJ_ERR_CUDA;
  return AJ_OK;
}

int32_t aj_nn_backward(int32_t n, int32_t h, int32_t w, const float* dy, const uint16_t* packed,
                       const float* master, void* act, size_t act_bytes, float* grad,
                       void* stream) {
  if (!nn_shape_ok(n, h, w) || !dy || !packed || !master || !act || !grad) return AJ_ERR_PARAM;
  conv_attrs();
  NnActs A = act_layout(n, h, w, act);
  if (act_bytes < A.total) return AJ_ERR_WORKSPACE;
  NnW W{reinterpret_cast<const __nv_bfloat16*>(packed), master};
  return nn_backward(n, h, w, dy, W, A, grad, (cudaStream_t)stream);
}

int32_t aj_nn_loss(int32_t n, int32_t h, int32_t w, const float* y, const float* target, float* dy,
                   double* loss, void* stream) {
  if (!nn_shape_ok(n, h, w) || !y || !target || !dy || !loss) return AJ_ERR_PARAM;
  cudaStream_t st = (cudaStream_t)stream;
  if (cudaMemsetAsync(loss, 0, sizeof(double), st) != cudaSuccess) return AJ_ERR_CUDA;
  const long P = (long)n * h * w;
  unsigned nb = cdiv(P, 256 * 4);
  if (nb > 1216) nb = 1216;
  k_mse<<<nb, 256, 0, st>>>(y, target, dy, P, loss);
  return cudaGetLastError() == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
}

int32_t aj_nn_expand(int32_t n, int32_t h, int32_t w, const float* x3, float* x16, void* stream) {
  if (!nn_shape_ok(n, h, w) || !x3 || !x16) return AJ_ERR_PARAM;
  const long cells = (long)n * h * w;
  k_nn_expand<<<cdiv(cells * 16, 256), 256, 0, (cudaStream_t)stream>>>(x3, x16, cells);
  return cudaGetLastError() == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
}

int32_t aj_nn_features(const AjStepParams* prm, const float* b, const float* mask,
                       const float* p_prev, const float* p_true, float* x3_out, float* target_out,
                       void* ws, size_t ws_bytes, void* stream) {
  if (!prm || !b || !mask || !p_prev || prm->nn_factor <= 0) return AJ_ERR_PARAM;
  Layout L;
  if (!make_layout(*prm, L) || !nn_step_shape_ok(*prm)) return AJ_ERR_SHAPE;
  if (!ws || ws_bytes < L.total) return AJ_ERR_WORKSPACE;
  const int F = prm->nn_factor;
  NnActs A = act_layout(1, prm->nx / F, prm->ny / F, at<char>(ws, L.nn_act));
  return nn_features(*prm, ws, at<double>(ws, L.part), b, mask, p_prev, p_true, A.x, x3_out,
                     target_out, (cudaStream_t)stream, false, true);
}

int32_t aj_nn_warmstart(const AjStepParams* prm, const float* rhs, const float* mask,
                        const float* p_prev, const uint16_t* nn_packed, const float* nn_master,
                        float* p0, void* ws, size_t ws_bytes, void* stream) {
  if (!prm || !rhs || !mask || !p_prev || !nn_packed || !nn_master || !p0) return AJ_ERR_PARAM;
  const AjStepParams p = normalise(*prm);
  if (p.nn_factor <= 0 || p.mg_mode != AJ_MG_CONVERGE) return AJ_ERR_PARAM;
  Layout L;
  if (!make_layout(p, L) || !nn_step_shape_ok(p)) return AJ_ERR_SHAPE;
  if (!ws || ws_bytes < L.total || !L.nn_act) return AJ_ERR_WORKSPACE;
  conv_attrs();
  const cudaStream_t st = (cudaStream_t)stream;
  DevScalars* sc = at<DevScalars>(ws, 0);
  // the scale reduction's last-block counter starts at zero (a workspace
  // that no step has used yet holds anything)
  if (cudaMemsetAsync(&sc->red_count, 0, sizeof(sc->red_count), st) != cudaSuccess)
    return AJ_ERR_CUDA;
  const int F = p.nn_factor, h = p.nx / F, w = p.ny / F;
  NnActs A = act_layout(1, h, w, at<char>(ws, L.nn_act));
  int rc = nn_features(p, ws, at<double>(ws, L.part), rhs, mask, p_prev, nullptr, A.x, nullptr,
                       nullptr, st, false, false);
  if (rc != AJ_OK) return rc;
  const NnW W{reinterpret_cast<const __nv_bfloat16*>(nn_packed), nn_master};
  rc = nn_forward(1, h, w, W, A, st, false, sc);
  if (rc != AJ_OK) return rc;
  const dim3 blk(32, 8), grd(cdiv(p.ny, 32), cdiv(p.nx, 8));
  launch_pdl(true, k_nn_apply_guess, grd, blk, 0, st, (const float*)A.y, p.nx, p.ny, F, p_prev, p0,
             (const DevScalars*)sc);
  return cudaGetLastError() == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
}

int32_t aj_nn_adam(float* master, const float* grad, float* m, float* v, int32_t step, float lr,
                   float beta1, float beta2, float eps, float clip, void* stream) {
  if (!master || !grad || !m || !v || step < 1) return AJ_ERR_PARAM;
  const long n = (long)n_params();
  const float c1 = (float)(1.0 / (1.0 - pow((double)beta1, step)));
  const float c2 = (float)(1.0 / (1.0 - pow((double)beta2, step)));
  k_adam<<<cdiv(n, 256), 256, 0, (cudaStream_t)stream>>>(master, grad, m, v, n, lr, beta1, beta2,
                                                         eps, clip, c1, c2);
  return cudaGetLastError() == cudaSuccess ? AJ_OK : AJ_ERR_CUDA;
}

}  // extern "C"
