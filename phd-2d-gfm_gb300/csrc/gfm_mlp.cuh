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
  g.gated = c_gt(ratio, 0.0) && c_gt(fabs(gfm_log(ratio)), MLP_GATE);
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

__host__ __device__ inline float mlp_silu(float z) { return z / (1.0f + expf(-z)); }

#if defined(__CUDACC__)
// The network in FP32 by one warp (all 32 lanes, warp-uniform): lane l
// computes neurons l and l + 32 of each layer from the parameters P in
// global memory; hbuf holds a layer's 64 outputs (per-warp shared memory).
__device__ inline float mlp_forward_warp(const float* __restrict__ P, const float x[MLP_IN], float* hbuf) {
  const int l = threadIdx.x & 31;
  float z0 = __ldg(P + MLP_B1 + l), z1 = __ldg(P + MLP_B1 + l + 32);
  for (int k = 0; k < MLP_IN; k++) {
    z0 += x[k] * __ldg(P + MLP_W1 + k * MLP_H + l);
    z1 += x[k] * __ldg(P + MLP_W1 + k * MLP_H + l + 32);
  }
  for (int layer = 0; layer < 2; layer++) {
    __syncwarp();
    hbuf[l] = mlp_silu(z0);
    hbuf[l + 32] = mlp_silu(z1);
    __syncwarp();
    const float* W = P + (layer == 0 ? MLP_W2 : MLP_W3);
    const float* b = P + (layer == 0 ? MLP_B2 : MLP_B3);
    z0 = __ldg(b + l);
    z1 = __ldg(b + l + 32);
    for (int k = 0; k < MLP_H; k++) {
      const float h = hbuf[k];
      z0 += h * __ldg(W + k * MLP_H + l);
      z1 += h * __ldg(W + k * MLP_H + l + 32);
    }
  }
  float y = mlp_silu(z0) * __ldg(P + MLP_W4 + l) + mlp_silu(z1) * __ldg(P + MLP_W4 + l + 32);
  for (int o = 16; o > 0; o >>= 1) y += __shfl_xor_sync(0xffffffffu, y, o);
  return y + __ldg(P + MLP_B4);
}
#endif

// counter-based generator (splitmix64 finaliser): uniform in [0, 1)
__host__ __device__ inline uint64_t mlp_mix(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__host__ __device__ inline double mlp_uniform(uint64_t seed, uint64_t k) {
  return (double)(mlp_mix(seed ^ mlp_mix(k)) >> 11) * 0x1p-53;
}

}  // namespace gfm
