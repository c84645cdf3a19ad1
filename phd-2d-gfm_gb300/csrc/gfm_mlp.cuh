// Learned star-pressure proposal for the exact Riemann solver.
//
// A multilayer perceptron 10 -> 64 -> 64 -> 64 -> 1 (SiLU) reads the
// normalised states of a Riemann problem,
//   x0,x1  log(rho_K / rho_ref)         rho_ref = max(rho_L, rho_R)
//   x2,x3  (u_K - (u_L+u_R)/2) / c_ref  c_ref = sqrt(p_ref / rho_ref)
//   x4,x5  log((p_K + pinf_K) / p_ref)  p_ref = max(p_L + pinf_L, p_R + pinf_R)
//   x6,x7  (gamma_K - 2.7) / 1.7
//   x8,x9  pinf_K / p_ref
// and outputs the logarithm of the star pressure relative to the solver's
// two-shock guess: y = log((p* + pinf_min) / (p_TSRS + pinf_min)).  The
// correction is applied only where the two-shock guess moved far from the
// PVRS guess (|log((p_TSRS + pinf_min)/(p_PVRS' + pinf_min))| > 1e-2, strong
// waves); elsewhere the two-shock guess is already within about 1e-6 and is
// kept.  Newton's method then runs from the proposal exactly as from any
// other guess, so the converged p* meets the same tolerance and the exact
// solver has the last word.
#pragma once

#include "gfm_math.cuh"

#if defined(__CUDACC__)
#include <cuda_bf16.h>
#endif

namespace gfm {

constexpr int MLP_IN = 10;
constexpr int MLP_H = 64;
// parameter offsets (floats): W1[10][64] b1[64] W2[64][64] b2[64] W3[64][64] b3[64] w4[64] b4
constexpr int MLP_W1 = 0;
constexpr int MLP_B1 = MLP_W1 + MLP_IN * MLP_H;
constexpr int MLP_W2 = MLP_B1 + MLP_H;
constexpr int MLP_B2 = MLP_W2 + MLP_H * MLP_H;
constexpr int MLP_W3 = MLP_B2 + MLP_H;
constexpr int MLP_B3 = MLP_W3 + MLP_H * MLP_H;
constexpr int MLP_W4 = MLP_B3 + MLP_H;
constexpr int MLP_B4 = MLP_W4 + MLP_H;
constexpr int MLP_NPARAM = MLP_B4 + 1;   // 9089

constexpr double MLP_GATE = 1e-2;
// The gate |gfm_log(ratio)| > MLP_GATE as two comparisons, without the
// logarithm: MLP_GATE_HI is the least double whose gfm_log exceeds 1e-2 and
// MLP_GATE_LO the greatest double whose gfm_log is below -1e-2 (gfm_log is
// monotone there; tests/gate_check.cpp checks both against gfm_log).
constexpr double MLP_GATE_HI = 0x1.0292a5d2f2227p+0;   // 1.0100501670841682
constexpr double MLP_GATE_LO = 0x1.fae7cfd2b9cfdp-1;   // 0.9900498337491680
GFM_HD bool mlp_gated(double ratio) {
  return c_le(MLP_GATE_HI, ratio) || (c_gt0(ratio) && c_le(ratio, MLP_GATE_LO));
}

// Guesses and features of one Riemann problem given its sides (rho, u, p)
// and gases; the PVRS guess is floored as rs_star floors its start.
struct GuessInfo {
  double ppv_f;      // max(PVRS, floor)
  double pts;        // two-shock guess at ppv_f
  double qmin;       // min(pinf_L, pinf_R)
  bool gated;        // the learned correction applies
};

GFM_HD GuessInfo rs_guess_info(const RSSide& L, const Gas& kL, const RSSide& R, const Gas& kR) {
  GuessInfo g;
  const double ppv = rs_guess_pvrs(L, R);
  g.qmin = c_lt(kL.pinf, kR.pinf) ? kL.pinf : kR.pinf;
  const double pbmin = c_lt(L.pb, R.pb) ? L.pb : R.pb;
  const double pfl = 1e-6 * pbmin - g.qmin;
  g.ppv_f = c_gt(ppv, pfl) ? ppv : pfl;
  g.pts = rs_guess_tsrs(L, kL, R, kR, g.ppv_f);
  const double ratio = (g.pts + g.qmin) / (g.ppv_f + g.qmin);
  g.gated = mlp_gated(ratio);
  return g;
}

// the ten input features, computed in float (velocity jump in double)
GFM_HD void mlp_features_f(double rhoL, double uL, double pbL, double gL, double qL, double rhoR, double uR,
                           double pbR, double gR, double qR, float x[MLP_IN]) {
  const float rl = (float)rhoL, rr = (float)rhoR, pl = (float)pbL, pr = (float)pbR;
  const float rref = fmaxf(rl, rr), pref = fmaxf(pl, pr);
  const float cref = sqrtf(pref / rref);
  const float half_jump = (float)(0.5 * (uR - uL)) / cref;
  x[0] = logf(rl / rref);
  x[1] = logf(rr / rref);
  x[2] = -half_jump;
  x[3] = half_jump;
  x[4] = logf(pl / pref);
  x[5] = logf(pr / pref);
  x[6] = ((float)gL - 2.7f) / 1.7f;
  x[7] = ((float)gR - 2.7f) / 1.7f;
  x[8] = (float)qL / pref;
  x[9] = (float)qR / pref;
}
GFM_HD void mlp_features(const RSSide& L, const Gas& kL, const RSSide& R, const Gas& kR, float x[MLP_IN]) {
  mlp_features_f(L.rho, L.u, L.pb, kL.g, kL.pinf, R.rho, R.u, R.pb, kR.g, kR.pinf, x);
}

// start of Newton given the network's output y for a gated problem
GFM_HD double mlp_apply(const GuessInfo& g, float y) {
  const float yc = fminf(fmaxf(y, -20.0f), 20.0f);
  return (g.pts + g.qmin) * gfm_exp((double)yc) - g.qmin;
}

GFM_HD float mlp_silu(float z) { return z / (1.0f + expf(-z)); }

#if defined(__CUDACC__)
// The network on the tensor cores by one warp, for one problem at a time
// inside the latency-bound interface loop.  Each layer is a row of 16 x 16
// BF16 tiles times the weights, D = A B + C with
// mma.sync.m16n8k16.row.col.f32.bf16.bf16.f32: the problem is row 0 of A
// (rows 1-15 zero), C starts at the bias, FP32 accumulation.  In this shape
// row 0 of D sits in lanes 0-3 (columns 8t + 2l, 8t + 2l + 1 of n-tile t),
// exactly where the next layer's A fragments need it (k-step s takes n-tiles
// 2s and 2s + 1), so the activations never leave their lanes.  The last
// layer (64 -> 1) is an FP32 dot product over lanes 0-3.  B fragments come
// pre-arranged per lane (MLP_FRAG_WORDS words, k_mlp_frag_pack): for layer L,
// k-step s, n-tile t, lane l the two words at ((MLP_FRAG_OFF[L] + 8 s + t) 32
// + l) 2 hold W[16 s + 2 (l & 3) + {0, 1}][8 t + (l >> 2)] and the same rows
// + 8, BF16 pairs with the lower k in the low half.
constexpr int MLP_FRAG_TILES = 8 + 32 + 32;           // (k-step, n-tile) pairs of the three layers
constexpr int MLP_FRAG_WORDS = MLP_FRAG_TILES * 64;   // 32 lanes x 2 words each

__device__ __forceinline__ uint32_t mlp_bf16x2(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&v);
}

__device__ __forceinline__ void mlp_mma(float c[4], uint32_t a0, uint32_t a2, uint2 b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
      "{%0, %1, %2, %3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(0u), "r"(a2), "r"(0u), "r"(b.x), "r"(b.y));
}

// the network's output for the warp's problem x (all lanes hold the same x);
// every lane returns it
__device__ inline float mlp_forward_warp_tc(const uint32_t* __restrict__ frag, const float* __restrict__ P,
                                            const float x[MLP_IN]) {
  const int lane = threadIdx.x & 31;
  const int tig = lane & 3;
  const bool row0 = lane < 4;
  const uint2* F = reinterpret_cast<const uint2*>(frag) + lane;
  float h[8][2];   // row 0 of the layer's output: columns 8 t + 2 tig + {0, 1} (lanes 0-3)
  // layer 1: K = 10 features padded to 16
  uint32_t a0 = 0u, a2 = 0u;
  if (row0) {
    a0 = mlp_bf16x2(x[2 * tig], x[2 * tig + 1]);
    a2 = tig == 0 ? mlp_bf16x2(x[8], x[9]) : 0u;
  }
#pragma unroll
  for (int t = 0; t < 8; t++) {
    float c[4] = {row0 ? __ldg(P + MLP_B1 + 8 * t + 2 * tig) : 0.0f,
                  row0 ? __ldg(P + MLP_B1 + 8 * t + 2 * tig + 1) : 0.0f, 0.0f, 0.0f};
    mlp_mma(c, a0, a2, __ldg(F + 32 * t));
    h[t][0] = c[0];
    h[t][1] = c[1];
  }
  // layers 2 and 3: K = 64 in four k-steps
#pragma unroll
  for (int layer = 0; layer < 2; layer++) {
    uint32_t A0[4], A2[4];
#pragma unroll
    for (int s = 0; s < 4; s++) {
      A0[s] = row0 ? mlp_bf16x2(mlp_silu(h[2 * s][0]), mlp_silu(h[2 * s][1])) : 0u;
      A2[s] = row0 ? mlp_bf16x2(mlp_silu(h[2 * s + 1][0]), mlp_silu(h[2 * s + 1][1])) : 0u;
    }
    const float* b = P + (layer == 0 ? MLP_B2 : MLP_B3);
    const uint2* FL = F + 32 * (8 + 32 * layer);
#pragma unroll
    for (int t = 0; t < 8; t++) {
      float c[4] = {row0 ? __ldg(b + 8 * t + 2 * tig) : 0.0f, row0 ? __ldg(b + 8 * t + 2 * tig + 1) : 0.0f, 0.0f,
                    0.0f};
#pragma unroll
      for (int s = 0; s < 4; s++) mlp_mma(c, A0[s], A2[s], __ldg(FL + 32 * (8 * s + t)));
      h[t][0] = c[0];
      h[t][1] = c[1];
    }
  }
  // output layer in FP32 over row 0's 64 activations (lanes 0-3)
  float y = 0.0f;
#pragma unroll
  for (int t = 0; t < 8; t++)
    y += mlp_silu(h[t][0]) * __ldg(P + MLP_W4 + 8 * t + 2 * tig) +
         mlp_silu(h[t][1]) * __ldg(P + MLP_W4 + 8 * t + 2 * tig + 1);
  y += __shfl_xor_sync(0xffffffffu, y, 1);
  y += __shfl_xor_sync(0xffffffffu, y, 2);
  return __shfl_sync(0xffffffffu, y, 0) + __ldg(P + MLP_B4);
}

// B fragments of the three layers from the FP32 parameters (one word per thread)
__global__ void k_mlp_frag_pack(const float* __restrict__ P, uint32_t* __restrict__ frag);
#endif

// counter-based generator (splitmix64 finaliser): uniform in [0, 1)
GFM_HD uint64_t mlp_mix(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
GFM_HD double mlp_uniform(uint64_t seed, uint64_t k) {
  return (double)(mlp_mix(seed ^ mlp_mix(k)) >> 11) * 0x1p-53;
}

}  // namespace gfm
