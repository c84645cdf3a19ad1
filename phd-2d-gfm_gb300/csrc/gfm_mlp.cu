// Learned star-pressure proposal (gfm_mlp.cuh): training problems from the
// exact solver, hand-written FP32 training kernels (forward, backward, Adam),
// and inference -- FP32 on the CUDA cores as the reference, BF16 on the
// tensor cores (tcgen05.mma, FP32 accumulators in tensor memory) for use --
// plus the batched two-material Riemann solve with the proposal fused in.
#include "gfm_internal.cuh"
#include "gfm_mlp.cuh"
#include <cstdio>
#include <cstring>
#include <vector>

namespace gfm {

// ---------------------------------------------------------------------------
// Training problems: the distribution of the learned-guess configuration
//   gamma_L,R ~ U[1.09, 4.4], pinf_L,R in {0, 6e8}, p_L ~ 10^U[3,8],
//   p_R / p_L ~ log-U[1e-3, 1e5], rho_L ~ 10^U[-1,3], rho_R / rho_L ~
//   log-U[1e-3, 1e3], u_R - u_L ~ U[-3, 3] (c_L + c_R)/2;
// problems that generate vacuum or do not pass the gate are skipped; the
// target comes from the exact solver (Newton from the two-shock guess).
// ---------------------------------------------------------------------------
__global__ void k_mlp_generate(uint64_t seed, uint64_t base, int n_try, float* X, float* Y, int cap, int* count) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n_try; k += gridDim.x * blockDim.x) {
    const uint64_t id = (base + (uint64_t)k) * 16ull;
    auto U = [&](int j) { return mlp_uniform(seed, id + (uint64_t)j); };
    const double ln10 = 2.302585092994045684;
    const double gL = 1.09 + 3.31 * U(0), gR = 1.09 + 3.31 * U(1);
    const double qL = U(2) < 0.5 ? 0.0 : 6e8, qR = U(3) < 0.5 ? 0.0 : 6e8;
    const double pL = gfm_exp((3.0 + 5.0 * U(4)) * ln10);
    const double pR = pL * gfm_exp(-3.0 * ln10 + 8.0 * ln10 * U(5));
    const double rL = gfm_exp((-1.0 + 4.0 * U(6)) * ln10);
    const double rR = rL * gfm_exp(-3.0 * ln10 + 6.0 * ln10 * U(7));
    const Gas kL = make_gas(gL, qL), kR = make_gas(gR, qR);
    RSSide L = rs_side(rL, 0.0, pL, kL), R = rs_side(rR, 0.0, pR, kR);
    rs_side_consts(L, kL);
    rs_side_consts(R, kR);
    const double du = (6.0 * U(8) - 3.0) * 0.5 * (L.c + R.c);
    L.u = -0.5 * du;
    R.u = 0.5 * du;
    if (c_le(L.G4c + R.G4c, R.u - L.u)) continue;   // vacuum
    const GuessInfo g = rs_guess_info(L, kL, R, kR);
    if (!g.gated) continue;
    const RSStar s = rs_star(L, kL, R, kR, g.pts);
    if (s.status != ST_OK) continue;
    const double y = gfm_log((s.p + g.qmin) / (g.pts + g.qmin));
    if (!(fabs(y) < 30.0)) continue;
    float x[MLP_IN];
    mlp_features(L, kL, R, kR, x);
    const int slot = atomicAdd(count, 1);
    if (slot >= cap) continue;
    for (int q = 0; q < MLP_IN; q++) X[(int64_t)slot * MLP_IN + q] = x[q];
    Y[slot] = (float)y;
  }
}

// ---------------------------------------------------------------------------
// Training: one CTA per chunk of 64 samples of a minibatch of B; forward
// pass and backward pass in shared memory, chunk gradients added to G.
// Loss = mean over the minibatch of (y - target)^2.
// ---------------------------------------------------------------------------
constexpr int TCH = 64;   // samples per chunk
constexpr int TNT = 256;  // threads

struct TrainSmem {
  float w[MLP_NPARAM + 3];
  float x[TCH][MLP_IN];
  float t[TCH];
  float z1[TCH][MLP_H], z2[TCH][MLP_H], z3[TCH][MLP_H];
  float da[TCH][MLP_H], db[TCH][MLP_H];
  float dy[TCH];
  float loss[TNT / 32];
};

__device__ __forceinline__ float sig(float z) { return 1.0f / (1.0f + expf(-z)); }
__device__ __forceinline__ float silu_d(float z) { const float s = sig(z); return s * (1.0f + z * (1.0f - s)); }

__global__ void __launch_bounds__(TNT) k_mlp_grad(const float* P, const float* X, const float* Y, const int* order,
                                                  int start, int B, float* G, float* loss) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TrainSmem& s = *reinterpret_cast<TrainSmem*>(smem_raw);
  const int tid = threadIdx.x, j = tid % MLP_H, r = tid / MLP_H;   // r in 0..3
  const int c0 = blockIdx.x * TCH;
  for (int k = tid; k < MLP_NPARAM; k += TNT) s.w[k] = P[k];
  for (int k = tid; k < TCH * MLP_IN; k += TNT) {
    const int sm = k / MLP_IN, q = k % MLP_IN;
    const int b = c0 + sm;
    s.x[sm][q] = (b < B) ? X[(int64_t)order[start + b] * MLP_IN + q] : 0.0f;
  }
  for (int sm = tid; sm < TCH; sm += TNT) s.t[sm] = (c0 + sm < B) ? Y[order[start + c0 + sm]] : 0.0f;
  __syncthreads();
  const float* W1 = s.w + MLP_W1;
  const float* W2 = s.w + MLP_W2;
  const float* W3 = s.w + MLP_W3;
  // forward: z[s][j] for samples s = r, r+4, ...
  for (int sm = r; sm < TCH; sm += 4) {
    float a = s.w[MLP_B1 + j];
    for (int k = 0; k < MLP_IN; k++) a += s.x[sm][k] * W1[k * MLP_H + j];
    s.z1[sm][j] = a;
  }
  __syncthreads();
  for (int sm = r; sm < TCH; sm += 4) {
    float a = s.w[MLP_B2 + j];
    for (int k = 0; k < MLP_H; k++) a += mlp_silu(s.z1[sm][k]) * W2[k * MLP_H + j];
    s.z2[sm][j] = a;
  }
  __syncthreads();
  for (int sm = r; sm < TCH; sm += 4) {
    float a = s.w[MLP_B3 + j];
    for (int k = 0; k < MLP_H; k++) a += mlp_silu(s.z2[sm][k]) * W3[k * MLP_H + j];
    s.z3[sm][j] = a;
  }
  __syncthreads();
  // output and its error: one warp per 32 samples
  float lsum = 0.0f;
  if (tid < TCH) {
    const int sm = tid;
    float yv = s.w[MLP_B4];
    for (int k = 0; k < MLP_H; k++) yv += mlp_silu(s.z3[sm][k]) * s.w[MLP_W4 + k];
    const bool valid = c0 + sm < B;
    const float e = valid ? yv - s.t[sm] : 0.0f;
    s.dy[sm] = 2.0f * e / (float)B;
    lsum = e * e;
  }
  for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
  if ((tid & 31) == 0) s.loss[tid >> 5] = lsum;
  __syncthreads();
  if (tid == 0) {
    float l = 0.0f;
    for (int q = 0; q < TNT / 32; q++) l += s.loss[q];
    atomicAdd(loss, l);
  }
  // layer 4: g_w4[k] = sum_s silu(z3) dy ; g_b4 = sum dy ; da = dy w4 silu'(z3)
  if (tid < MLP_H) {
    float gw = 0.0f;
    for (int sm = 0; sm < TCH; sm++) gw += mlp_silu(s.z3[sm][tid]) * s.dy[sm];
    atomicAdd(&G[MLP_W4 + tid], gw);
  }
  if (tid == MLP_H) {
    float gb = 0.0f;
    for (int sm = 0; sm < TCH; sm++) gb += s.dy[sm];
    atomicAdd(&G[MLP_B4], gb);
  }
  for (int sm = r; sm < TCH; sm += 4) s.da[sm][j] = s.dy[sm] * s.w[MLP_W4 + j] * silu_d(s.z3[sm][j]);
  __syncthreads();
  // layer 3: g_W3[k][j] = sum_s silu(z2[s][k]) da[s][j]; db = (da W3^T) silu'(z2)
  for (int k = r; k < MLP_H; k += 4) {
    float gw = 0.0f;
    for (int sm = 0; sm < TCH; sm++) gw += mlp_silu(s.z2[sm][k]) * s.da[sm][j];
    atomicAdd(&G[MLP_W3 + k * MLP_H + j], gw);
  }
  if (tid < MLP_H) {
    float gb = 0.0f;
    for (int sm = 0; sm < TCH; sm++) gb += s.da[sm][tid];
    atomicAdd(&G[MLP_B3 + tid], gb);
  }
  for (int sm = r; sm < TCH; sm += 4) {
    float a = 0.0f;
    for (int q = 0; q < MLP_H; q++) a += s.da[sm][q] * W3[j * MLP_H + q];
    s.db[sm][j] = a * silu_d(s.z2[sm][j]);
  }
  __syncthreads();
  // layer 2
  for (int k = r; k < MLP_H; k += 4) {
    float gw = 0.0f;
    for (int sm = 0; sm < TCH; sm++) gw += mlp_silu(s.z1[sm][k]) * s.db[sm][j];
    atomicAdd(&G[MLP_W2 + k * MLP_H + j], gw);
  }
  if (tid < MLP_H) {
    float gb = 0.0f;
    for (int sm = 0; sm < TCH; sm++) gb += s.db[sm][tid];
    atomicAdd(&G[MLP_B2 + tid], gb);
  }
  for (int sm = r; sm < TCH; sm += 4) {
    float a = 0.0f;
    for (int q = 0; q < MLP_H; q++) a += s.db[sm][q] * W2[j * MLP_H + q];
    s.da[sm][j] = a * silu_d(s.z1[sm][j]);
  }
  __syncthreads();
  // layer 1
  for (int k = r; k < MLP_IN; k += 4) {
    float gw = 0.0f;
    for (int sm = 0; sm < TCH; sm++) gw += s.x[sm][k] * s.da[sm][j];
    atomicAdd(&G[MLP_W1 + k * MLP_H + j], gw);
  }
  if (tid < MLP_H) {
    float gb = 0.0f;
    for (int sm = 0; sm < TCH; sm++) gb += s.da[sm][tid];
    atomicAdd(&G[MLP_B1 + tid], gb);
  }
}

// Adam step (bias-corrected), then the gradient accumulator is cleared.
__global__ void k_mlp_adam(float* P, float* G, float* M, float* V, float lr, float c1, float c2) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= MLP_NPARAM) return;
  const float g = G[k];
  const float m = 0.9f * M[k] + 0.1f * g;
  const float v = 0.999f * V[k] + 0.001f * g * g;
  M[k] = m;
  V[k] = v;
  P[k] -= lr * (m / c1) / (sqrtf(v / c2) + 1e-8f);
  G[k] = 0.0f;
}

// ---------------------------------------------------------------------------
// FP32 inference on the CUDA cores (the reference for the tensor-core path)
// ---------------------------------------------------------------------------
__device__ float mlp_forward_f32(const float* w, const float* x) {
  float h1[MLP_H], h2[MLP_H];
  for (int j = 0; j < MLP_H; j++) {
    float a = w[MLP_B1 + j];
    for (int k = 0; k < MLP_IN; k++) a += x[k] * w[MLP_W1 + k * MLP_H + j];
    h1[j] = mlp_silu(a);
  }
  for (int j = 0; j < MLP_H; j++) {
    float a = w[MLP_B2 + j];
    for (int k = 0; k < MLP_H; k++) a += h1[k] * w[MLP_W2 + k * MLP_H + j];
    h2[j] = mlp_silu(a);
  }
  float y = w[MLP_B4];
  for (int j = 0; j < MLP_H; j++) {
    float a = w[MLP_B3 + j];
    for (int k = 0; k < MLP_H; k++) a += h2[k] * w[MLP_W3 + k * MLP_H + j];
    y += mlp_silu(a) * w[MLP_W4 + j];
  }
  return y;
}

__global__ void k_mlp_infer_f32(const float* P, const float* X, int n, float* out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* w = reinterpret_cast<float*>(smem_raw);
  for (int k = threadIdx.x; k < MLP_NPARAM; k += blockDim.x) w[k] = P[k];
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float x[MLP_IN];
    for (int q = 0; q < MLP_IN; q++) x[q] = X[(int64_t)i * MLP_IN + q];
    out[i] = mlp_forward_f32(w, x);
  }
}

// ---------------------------------------------------------------------------
// Warp-level tensor-core inference (mlp_forward_warp_tc, the interface
// loop's path): its B fragments, and a batch kernel of one warp per problem
// that runs the same function for tests and measurements.
// ---------------------------------------------------------------------------
__global__ void k_mlp_frag_pack(const float* __restrict__ P, uint32_t* __restrict__ frag) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= MLP_FRAG_WORDS) return;
  const int tile = w >> 6, lane = (w >> 1) & 31, half = w & 1;
  int layer, ks, t;
  if (tile < 8) { layer = 0; ks = 0; t = tile; }
  else if (tile < 40) { layer = 1; ks = (tile - 8) >> 3; t = (tile - 8) & 7; }
  else { layer = 2; ks = (tile - 40) >> 3; t = (tile - 40) & 7; }
  const int n = 8 * t + (lane >> 2);
  const int k = 16 * ks + 2 * (lane & 3) + 8 * half;
  const int base = layer == 0 ? MLP_W1 : (layer == 1 ? MLP_W2 : MLP_W3);
  const int kmax = layer == 0 ? MLP_IN : MLP_H;
  const float lo = k < kmax ? P[base + k * MLP_H + n] : 0.0f;
  const float hi = k + 1 < kmax ? P[base + (k + 1) * MLP_H + n] : 0.0f;
  frag[w] = mlp_bf16x2(lo, hi);
}

__global__ void __launch_bounds__(128) k_mlp_infer_warp_tc(const uint32_t* frag, const float* P, const float* X,
                                                           int n, float* out) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int q = warp; q < n; q += nwarps) {
    float x[MLP_IN];
    for (int k = 0; k < MLP_IN; k++) x[k] = X[(int64_t)q * MLP_IN + k];
    const float y = mlp_forward_warp_tc(frag, P, x);
    if ((threadIdx.x & 31) == 0) out[q] = y;
  }
}

// ---------------------------------------------------------------------------
// BF16 inference on the tensor cores.
//
// One CTA of 128 threads per tile of 128 problems (thread t = row t).  Each
// layer is D[128 x 64] = A[128 x K] B[K x 64] with tcgen05.mma (kind::f16,
// BF16 operands, FP32 accumulator in tensor memory, 64 columns allocated
// once per CTA), issued by thread 0 and completed on an mbarrier; every
// thread then reads its row of D (tcgen05.ld 32x32b), adds the bias, applies
// SiLU and writes the next layer's A row in BF16.  The first layer's K is
// the 10 features padded to 16; the last layer (64 -> 1) runs in FP32.
//
// Operands sit in shared memory in the canonical K-major layout without
// swizzling: 8-row x 16-byte core matrices of 128 contiguous bytes,
//   byte(r, k) = (r/8) SBO + (k/8) LBO + (r%8) 16 + (k%8) 2,
// LBO = 128 (next core matrix along K), SBO = (K/8) 128 (next 8 rows).
// Weights are packed in this layout (B stored as N x K) by the host.
// ---------------------------------------------------------------------------
constexpr int TC_M = 128;
constexpr int TC_K1 = 16;
constexpr uint32_t TC_TMEM_COLS = 64;
constexpr long long TC_SPIN_LIMIT = 1ll << 22;

// packed BF16 weights: B1 (64 x 16), B2 (64 x 64), B3 (64 x 64)
constexpr int TC_B1_ELEMS = MLP_H * TC_K1;
constexpr int TC_B2_ELEMS = MLP_H * MLP_H;
constexpr int TC_PACK_ELEMS = TC_B1_ELEMS + 2 * TC_B2_ELEMS;

__host__ __device__ inline int tc_offset(int r, int k, int K) {   // element offset in the canonical layout
  return (r / 8) * (K / 8) * 64 + (k / 8) * 64 + (r % 8) * 8 + (k % 8);
}

__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);   // version 1, no swizzle
}

// kind::f16, D = F32, A = B = BF16, both K-major, N = 64, M = 128
constexpr uint32_t TC_IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(MLP_H >> 3) << 17) |
                              ((uint32_t)(TC_M >> 4) << 24);

__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(TC_IDESC), "r"(accumulate));
}

__device__ __forceinline__ void tc_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

// bounded wait for the mbarrier phase with the given parity
__device__ __forceinline__ bool tc_wait(uint32_t mbar, uint32_t parity) {
  for (long long it = 0; it < TC_SPIN_LIMIT; it++) {
    uint32_t done;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done) : "r"(mbar), "r"(parity) : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void tc_ld16(uint32_t taddr, float v[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
  for (int q = 0; q < 16; q++) v[q] = __uint_as_float(r[q]);
}

__device__ __forceinline__ uint16_t bf16_bits(float f) {   // round to nearest even
  uint32_t u = __float_as_uint(f);
  if ((u & 0x7fffffffu) > 0x7f800000u) return 0x7fc0;
  u += 0x7fffu + ((u >> 16) & 1u);
  return (uint16_t)(u >> 16);
}

struct TcSmem {
  uint16_t b1[TC_B1_ELEMS];
  uint16_t b2[TC_B2_ELEMS];
  uint16_t b3[TC_B2_ELEMS];
  uint16_t a0[TC_M * TC_K1];
  uint16_t a1[TC_M * MLP_H];
  float bias[3][MLP_H];
  float w4[MLP_H];
  float b4;
  unsigned long long mbar;
  uint32_t tmem;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// rows of one tile through the three tensor-core layers; out[row] = y
__device__ void tc_tile(TcSmem& s, uint32_t tmem, uint32_t mbar, uint32_t& phase, int row_valid, float y_out[1],
                        const float x[MLP_IN], bool& ok) {
  const int t = threadIdx.x;
  const int w = t >> 5;
  const uint32_t tm_row = tmem + ((uint32_t)(w * 32) << 16);
  // layer-1 A row: the features in BF16, K padded to 16
  for (int k = 0; k < TC_K1; k++) s.a0[tc_offset(t, k, TC_K1)] = bf16_bits(k < MLP_IN ? x[k] : 0.0f);
  float y = s.b4;
  for (int layer = 0; layer < 3; layer++) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (t == 0) {
      if (layer == 0) {
        tc_mma(tmem, tc_desc(smem_u32(s.a0), 128, (TC_K1 / 8) * 128), tc_desc(smem_u32(s.b1), 128, (TC_K1 / 8) * 128), 0);
      } else {
        const uint16_t* B = (layer == 1) ? s.b2 : s.b3;
        for (int kk = 0; kk < MLP_H; kk += 16)
          tc_mma(tmem, tc_desc(smem_u32(s.a1) + (uint32_t)(kk / 8) * 128, 128, (MLP_H / 8) * 128),
                 tc_desc(smem_u32(B) + (uint32_t)(kk / 8) * 128, 128, (MLP_H / 8) * 128), kk > 0 ? 1u : 0u);
      }
      tc_commit(mbar);
    }
    const bool done = tc_wait(mbar, phase);
    phase ^= 1u;
    if (!__syncthreads_and(done)) {   // the MMA did not complete in time: issue nothing more
      ok = false;
      return;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // this thread's row of D: bias, SiLU; next A row (BF16) or the output
    for (int c = 0; c < MLP_H; c += 16) {
      float v[16];
      tc_ld16(tm_row + (uint32_t)c, v);
      for (int q = 0; q < 16; q++) {
        const float h = mlp_silu(v[q] + s.bias[layer][c + q]);
        if (layer < 2) s.a1[tc_offset(t, c + q, MLP_H)] = bf16_bits(h);
        else y += h * s.w4[c + q];
      }
    }
    // the MMA of the next layer overwrites D and reads a1: everyone is done
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  }
  (void)row_valid;
  y_out[0] = y;
}

__device__ bool tc_setup(TcSmem& s, const uint16_t* pack, const float* P, uint32_t& tmem, uint32_t& mbar) {
  const int t = threadIdx.x;
  for (int k = t; k < TC_B1_ELEMS; k += blockDim.x) s.b1[k] = pack[k];
  for (int k = t; k < TC_B2_ELEMS; k += blockDim.x) {
    s.b2[k] = pack[TC_B1_ELEMS + k];
    s.b3[k] = pack[TC_B1_ELEMS + TC_B2_ELEMS + k];
  }
  for (int k = t; k < MLP_H; k += blockDim.x) {
    s.bias[0][k] = P[MLP_B1 + k];
    s.bias[1][k] = P[MLP_B2 + k];
    s.bias[2][k] = P[MLP_B3 + k];
    s.w4[k] = P[MLP_W4 + k];
  }
  if (t == 0) s.b4 = P[MLP_B4];
  mbar = smem_u32(&s.mbar);
  if (t == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(1) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (t < 32) {   // warp 0 allocates (and later frees) the tensor memory
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s.tmem)),
                 "r"(TC_TMEM_COLS) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  tmem = s.tmem;
  return true;
}

// ok == false: the last committed MMA was not seen to complete; wait for it
// once more (bounded) before the tensor memory it writes is freed
__device__ void tc_teardown(uint32_t tmem, bool ok, uint32_t mbar, uint32_t phase) {
  if (!ok) tc_wait(mbar, phase ^ 1u);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (threadIdx.x < 32)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS) : "memory");
}

__global__ void __launch_bounds__(TC_M) k_mlp_infer_tc(const uint16_t* pack, const float* P, const float* X, int n,
                                                       float* out, int* err) {
  extern __shared__ __align__(128) unsigned char smem_tc[];
  TcSmem& s = *reinterpret_cast<TcSmem*>(smem_tc);
  uint32_t tmem, mbar, phase = 0;
  tc_setup(s, pack, P, tmem, mbar);
  bool ok = true;
  const int ntiles = (n + TC_M - 1) / TC_M;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int row = tile * TC_M + threadIdx.x;
    float x[MLP_IN];
    for (int q = 0; q < MLP_IN; q++) x[q] = row < n ? X[(int64_t)row * MLP_IN + q] : 0.0f;
    float y[1];
    tc_tile(s, tmem, mbar, phase, row < n, y, x, ok);
    if (row < n) out[row] = ok ? y[0] : 0.0f;
    if (!ok) break;   // an mbarrier wait ran out (ok is uniform across the CTA): stop issuing
  }
  if (!ok && threadIdx.x == 0) atomicOr(err, 1);
  tc_teardown(tmem, ok, mbar, phase);
}

// ---------------------------------------------------------------------------
// Batched two-material Riemann solve with the learned proposal: the same
// results as k_rs_mixed up to the start of Newton's method, which begins
// from the proposal for gated problems.  Per tile of 128 problems: sides,
// constants and guesses in FP64, features, the tensor-core network, then
// Newton (rs_star) and the star densities.
// out[4k..] = (p*, u*, rho*_L, rho*_R); iters[k] = Newton iterations.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(TC_M) k_rs_mixed_learned(const uint16_t* pack, const float* P, int n, Gas kL,
                                                           Gas kR, const double* UL, const double* UR, double* out,
                                                           int* iters, unsigned int* status, int use_net, int* err) {
  extern __shared__ __align__(128) unsigned char smem_tc[];
  TcSmem& s = *reinterpret_cast<TcSmem*>(smem_tc);
  uint32_t tmem = 0, mbar = 0, phase = 0;
  if (use_net) tc_setup(s, pack, P, tmem, mbar);
  bool ok = true;
  uint32_t st = 0;
  const int ntiles = (n + TC_M - 1) / TC_M;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int k = tile * TC_M + threadIdx.x;
    const bool valid = k < n;
    V4 ul{0, 0, 0, 0}, ur{0, 0, 0, 0};
    if (valid) {
      ul = V4{UL[4 * k], UL[4 * k + 1], UL[4 * k + 2], UL[4 * k + 3]};
      ur = V4{UR[4 * k], UR[4 * k + 1], UR[4 * k + 2], UR[4 * k + 3]};
    } else {
      ul = V4{1.0, 0.0, 0.0, 1.0};
      ur = ul;
    }
    bool okL, okR;
    V4 Lp = cons_to_prims_phys(kL.g, kL.pinf, ul, &okL);
    V4 Rp = cons_to_prims_phys(kR.g, kR.pinf, ur, &okR);
    if (valid && (!okL || !okR)) st |= ST_UNPHYSICAL;
    RSSide L = rs_side(Lp.a, Lp.b, Lp.d, kL), R = rs_side(Rp.a, Rp.b, Rp.d, kR);
    const bool trivial = c_eq(L.u, R.u) && c_eq(L.p, R.p);
    GuessInfo g;
    float x[MLP_IN];
    if (!trivial) {
      rs_side_consts(L, kL);
      rs_side_consts(R, kR);
      g = rs_guess_info(L, kL, R, kR);
      mlp_features(L, kL, R, kR, x);
    } else {
      g.gated = false; g.pts = 0.0; g.qmin = 0.0; g.ppv_f = 0.0;
      for (int q = 0; q < MLP_IN; q++) x[q] = 0.0f;
    }
    float y[1] = {0.0f};
    if (use_net) tc_tile(s, tmem, mbar, phase, valid, y, x, ok);   // every thread of the CTA takes part
    if (valid) {
      double ps, us, rl, rr;
      int it = 0;
      if (trivial) {
        ps = L.p; us = L.u; rl = L.rho; rr = R.rho;
      } else {
        const double p0 = (use_net && g.gated && ok) ? mlp_apply(g, y[0]) : g.pts;
        RSStar r = rs_star(L, kL, R, kR, p0);
        st |= r.status;
        ps = r.p; us = r.u; it = r.iters;
        rl = rs_rho_star(L, kL, ps);
        rr = rs_rho_star(R, kR, ps);
      }
      out[4 * k] = ps; out[4 * k + 1] = us; out[4 * k + 2] = rl; out[4 * k + 3] = rr;
      iters[k] = it;
    }
    if (use_net && !ok) break;   // uniform across the CTA
  }
  if (st) atomicOr(status, st);
  if (!ok && threadIdx.x == 0) atomicOr(err, 1);
  if (use_net) tc_teardown(tmem, ok, mbar, phase);
}

}  // namespace gfm

using namespace gfm;

struct gfm_mlp {
  float* P;          // parameters (FP32 master)
  float* G;          // gradient accumulator
  float* M;          // Adam moments
  float* V;
  uint16_t* pack;    // BF16 weights in the tensor-core layout
  uint32_t* frag;    // BF16 B fragments of the warp-level tensor-core path (mlp_forward_warp_tc)
  int* err;
  int adam_steps;
  bool pack_stale;
};

namespace {

gfm_status_t ck(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    fprintf(stderr, "gfm_mlp: %s: %s\n", what, cudaGetErrorString(e));
    return GFM_ERR_CUDA;
  }
  return GFM_OK;
}

uint16_t host_bf16(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  if ((u & 0x7fffffffu) > 0x7f800000u) return 0x7fc0;
  u += 0x7fffu + ((u >> 16) & 1u);
  return (uint16_t)(u >> 16);
}

// weights (K x 64, row k) -> B operand (64 x Kp) in the canonical layout
gfm_status_t repack(gfm_mlp* m, cudaStream_t s) {
  std::vector<float> P(MLP_NPARAM);
  if (cudaMemcpyAsync(P.data(), m->P, sizeof(float) * MLP_NPARAM, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return GFM_ERR_CUDA;
  std::vector<uint16_t> pack(TC_PACK_ELEMS, 0);
  for (int j = 0; j < MLP_H; j++) {
    for (int k = 0; k < TC_K1; k++)
      pack[tc_offset(j, k, TC_K1)] = host_bf16(k < MLP_IN ? P[MLP_W1 + k * MLP_H + j] : 0.0f);
    for (int k = 0; k < MLP_H; k++) {
      pack[TC_B1_ELEMS + tc_offset(j, k, MLP_H)] = host_bf16(P[MLP_W2 + k * MLP_H + j]);
      pack[TC_B1_ELEMS + TC_B2_ELEMS + tc_offset(j, k, MLP_H)] = host_bf16(P[MLP_W3 + k * MLP_H + j]);
    }
  }
  gfm_status_t r = ck(cudaMemcpyAsync(m->pack, pack.data(), sizeof(uint16_t) * TC_PACK_ELEMS,
                                      cudaMemcpyHostToDevice, s), "pack upload");
  if (r == GFM_OK) r = ck(cudaStreamSynchronize(s), "pack upload");
  if (r == GFM_OK) m->pack_stale = false;
  return r;
}

size_t tc_smem() { return sizeof(TcSmem); }

}  // namespace

const float* gfm::mlp_params(const gfm_mlp* m) { return m->P; }
const uint32_t* gfm::mlp_frag(const gfm_mlp* m) { return m->frag; }

// Stream-ordered, so a step recorded into a graph packs the network as it
// is when the step runs.
void gfm::launch_mlp_frag_pack(const gfm_mlp* m, cudaStream_t s) {
  k_mlp_frag_pack<<<(MLP_FRAG_WORDS + 255) / 256, 256, 0, s>>>(m->P, m->frag);
  counted();
}

extern "C" {

gfm_status_t gfm_mlp_create(uint64_t seed, gfm_mlp** out) {
  if (!out) return GFM_ERR_ARG;
  *out = nullptr;
  gfm_mlp* m = new gfm_mlp();
  memset(m, 0, sizeof(*m));
  cudaError_t e = cudaSuccess;
  e = cudaMalloc(&m->P, sizeof(float) * MLP_NPARAM);
  if (e == cudaSuccess) e = cudaMalloc(&m->G, sizeof(float) * MLP_NPARAM);
  if (e == cudaSuccess) e = cudaMalloc(&m->M, sizeof(float) * MLP_NPARAM);
  if (e == cudaSuccess) e = cudaMalloc(&m->V, sizeof(float) * MLP_NPARAM);
  if (e == cudaSuccess) e = cudaMalloc(&m->pack, sizeof(uint16_t) * TC_PACK_ELEMS);
  if (e == cudaSuccess) e = cudaMalloc(&m->frag, sizeof(uint32_t) * MLP_FRAG_WORDS);
  if (e == cudaSuccess) e = cudaMalloc(&m->err, sizeof(int));
  if (e != cudaSuccess) {
    gfm_mlp_destroy(m);
    return GFM_ERR_CUDA;
  }
  // He initialisation (normal via Box-Muller on the counter generator), zero biases
  std::vector<float> P(MLP_NPARAM, 0.0f);
  auto normal = [&](uint64_t k) {
    const double u1 = mlp_uniform(seed, 2 * k) + 1e-300, u2 = mlp_uniform(seed, 2 * k + 1);
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
  };
  uint64_t c = 0;
  for (int k = 0; k < MLP_IN * MLP_H; k++) P[MLP_W1 + k] = (float)(normal(c++) * std::sqrt(2.0 / MLP_IN));
  for (int k = 0; k < MLP_H * MLP_H; k++) P[MLP_W2 + k] = (float)(normal(c++) * std::sqrt(2.0 / MLP_H));
  for (int k = 0; k < MLP_H * MLP_H; k++) P[MLP_W3 + k] = (float)(normal(c++) * std::sqrt(2.0 / MLP_H));
  for (int k = 0; k < MLP_H; k++) P[MLP_W4 + k] = (float)(normal(c++) * std::sqrt(2.0 / MLP_H));
  gfm_status_t r = gfm_mlp_set_params(m, P.data());
  if (r != GFM_OK) {
    gfm_mlp_destroy(m);
    return r;
  }
  *out = m;
  return GFM_OK;
}

gfm_status_t gfm_mlp_destroy(gfm_mlp* m) {
  if (!m) return GFM_OK;
  cudaFree(m->P); cudaFree(m->G); cudaFree(m->M); cudaFree(m->V); cudaFree(m->pack); cudaFree(m->frag);
  cudaFree(m->err);
  delete m;
  return GFM_OK;
}

gfm_status_t gfm_mlp_set_params(gfm_mlp* m, const float* params) {
  if (!m || !params) return GFM_ERR_ARG;
  gfm_status_t r = ck(cudaMemcpy(m->P, params, sizeof(float) * MLP_NPARAM, cudaMemcpyHostToDevice), "set params");
  if (r == GFM_OK) r = ck(cudaMemset(m->G, 0, sizeof(float) * MLP_NPARAM), "clear");
  if (r == GFM_OK) r = ck(cudaMemset(m->M, 0, sizeof(float) * MLP_NPARAM), "clear");
  if (r == GFM_OK) r = ck(cudaMemset(m->V, 0, sizeof(float) * MLP_NPARAM), "clear");
  m->adam_steps = 0;
  m->pack_stale = true;
  return r;
}

gfm_status_t gfm_mlp_get_params(gfm_mlp* m, float* params) {
  if (!m || !params) return GFM_ERR_ARG;
  return ck(cudaMemcpy(params, m->P, sizeof(float) * MLP_NPARAM, cudaMemcpyDeviceToHost), "get params");
}

int gfm_mlp_param_count(void) { return MLP_NPARAM; }

gfm_status_t gfm_mlp_generate(uint64_t seed, int n, float* X, float* Y, int* n_out, void* cuda_stream) {
  if (n < 1 || !X || !Y || !n_out) return GFM_ERR_ARG;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(cuda_stream);
  int* count = nullptr;
  gfm_status_t r = ck(cudaMalloc(&count, sizeof(int)), "count");
  if (r != GFM_OK) return r;
  cudaMemsetAsync(count, 0, sizeof(int), s);
  int have = 0;
  uint64_t base = 0;
  for (int round = 0; round < 64 && have < n; round++) {
    const int tries = (n - have) * 2 + 65536;
    k_mlp_generate<<<(tries + 255) / 256, 256, 0, s>>>(seed, base, tries, X, Y, n, count);
    counted();
    base += (uint64_t)tries;
    if ((r = ck(cudaMemcpyAsync(&have, count, sizeof(int), cudaMemcpyDeviceToHost, s), "count")) != GFM_OK) break;
    if ((r = ck(cudaStreamSynchronize(s), "generate")) != GFM_OK) break;
  }
  cudaFree(count);
  *n_out = have < n ? have : n;
  return r;
}

gfm_status_t gfm_mlp_gradient(gfm_mlp* m, const float* X, const float* Y, int n, float* grad, float* loss,
                              void* cuda_stream) {
  if (!m || !X || !Y || n < 1 || !grad || !loss) return GFM_ERR_ARG;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(cuda_stream);
  int* order = nullptr;
  float* dloss = nullptr;
  std::vector<int> idx(n);
  for (int k = 0; k < n; k++) idx[k] = k;
  gfm_status_t r = ck(cudaMalloc(&order, sizeof(int) * n), "order");
  if (r == GFM_OK) r = ck(cudaMalloc(&dloss, sizeof(float)), "loss");
  if (r == GFM_OK) r = ck(cudaMemcpyAsync(order, idx.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s), "order");
  if (r == GFM_OK) {
    cudaMemsetAsync(m->G, 0, sizeof(float) * MLP_NPARAM, s);
    cudaMemsetAsync(dloss, 0, sizeof(float), s);
    cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TrainSmem));
    k_mlp_grad<<<(n + TCH - 1) / TCH, TNT, sizeof(TrainSmem), s>>>(m->P, X, Y, order, 0, n, m->G, dloss);
    counted();
    r = ck(cudaGetLastError(), "k_mlp_grad");
  }
  if (r == GFM_OK) r = ck(cudaMemcpyAsync(grad, m->G, sizeof(float) * MLP_NPARAM, cudaMemcpyDeviceToHost, s), "grad");
  if (r == GFM_OK) r = ck(cudaMemcpyAsync(loss, dloss, sizeof(float), cudaMemcpyDeviceToHost, s), "loss");
  if (r == GFM_OK) r = ck(cudaStreamSynchronize(s), "gradient");
  if (r == GFM_OK) {
    *loss /= (float)n;
    cudaMemsetAsync(m->G, 0, sizeof(float) * MLP_NPARAM, s);
  }
  cudaFree(order);
  cudaFree(dloss);
  return r;
}

gfm_status_t gfm_mlp_train(gfm_mlp* m, const float* X, const float* Y, int n, int epochs, int batch, float lr,
                           uint64_t seed, float* loss_per_epoch, void* cuda_stream) {
  if (!m || !X || !Y || n < batch || batch < 1 || epochs < 1 || !(lr > 0.0f)) return GFM_ERR_ARG;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(cuda_stream);
  int* order = nullptr;
  float* dloss = nullptr;
  gfm_status_t r = ck(cudaMalloc(&order, sizeof(int) * n), "order");
  if (r == GFM_OK) r = ck(cudaMalloc(&dloss, sizeof(float) * epochs), "loss");
  if (r != GFM_OK) {
    cudaFree(order);
    return r;
  }
  cudaMemsetAsync(dloss, 0, sizeof(float) * epochs, s);
  cudaMemsetAsync(m->G, 0, sizeof(float) * MLP_NPARAM, s);
  cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TrainSmem));
  std::vector<int> idx(n);
  for (int k = 0; k < n; k++) idx[k] = k;
  const int steps = n / batch;
  for (int ep = 0; ep < epochs && r == GFM_OK; ep++) {
    for (int k = n - 1; k > 0; k--) {   // Fisher-Yates with the counter generator
      const int q = (int)(mlp_uniform(seed + (uint64_t)ep, (uint64_t)k) * (double)(k + 1));
      const int t = idx[k]; idx[k] = idx[q]; idx[q] = t;
    }
    r = ck(cudaMemcpyAsync(order, idx.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s), "order");
    const float lr_ep = lr * 0.5f * (1.0f + std::cos(3.14159265f * (float)ep / (float)epochs));
    for (int st = 0; st < steps && r == GFM_OK; st++) {
      k_mlp_grad<<<(batch + TCH - 1) / TCH, TNT, sizeof(TrainSmem), s>>>(m->P, X, Y, order, st * batch, batch, m->G,
                                                                          dloss + ep);
      m->adam_steps++;
      const float c1 = 1.0f - std::pow(0.9f, (float)m->adam_steps), c2 = 1.0f - std::pow(0.999f, (float)m->adam_steps);
      k_mlp_adam<<<(MLP_NPARAM + 255) / 256, 256, 0, s>>>(m->P, m->G, m->M, m->V, lr_ep, c1, c2);
      counted(2);
    }
    if (r == GFM_OK) r = ck(cudaStreamSynchronize(s), "train epoch");   // idx is reused for the next epoch
  }
  if (r == GFM_OK && loss_per_epoch) {
    r = ck(cudaMemcpy(loss_per_epoch, dloss, sizeof(float) * epochs, cudaMemcpyDeviceToHost), "loss");
    for (int ep = 0; ep < epochs; ep++) loss_per_epoch[ep] /= (float)(steps * batch);
  }
  m->pack_stale = true;
  cudaFree(order);
  cudaFree(dloss);
  return r;
}

gfm_status_t gfm_mlp_infer(gfm_mlp* m, const float* X, int n, float* out, int tensor_cores, void* cuda_stream) {
  if (!m || !X || !out || n < 1) return GFM_ERR_ARG;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(cuda_stream);
  if (!tensor_cores) {
    const size_t sm = sizeof(float) * MLP_NPARAM;
    cudaFuncSetAttribute(k_mlp_infer_f32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_mlp_infer_f32<<<(n + 127) / 128, 128, sm, s>>>(m->P, X, n, out);
    counted();
    return ck(cudaGetLastError(), "k_mlp_infer_f32");
  }
  if (tensor_cores == 2) {   // the interface loop's warp-level path, one warp per problem
    launch_mlp_frag_pack(m, s);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = (n + 3) / 4 < sms * 16 ? (n + 3) / 4 : sms * 16;
    k_mlp_infer_warp_tc<<<blocks, 128, 0, s>>>(m->frag, m->P, X, n, out);
    counted();
    return ck(cudaGetLastError(), "k_mlp_infer_warp_tc");
  }
  if (m->pack_stale) {
    gfm_status_t r = repack(m, s);
    if (r != GFM_OK) return r;
  }
  cudaMemsetAsync(m->err, 0, sizeof(int), s);
  cudaFuncSetAttribute(k_mlp_infer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc_smem());
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int tiles = (n + TC_M - 1) / TC_M;
  k_mlp_infer_tc<<<tiles < sms * 4 ? tiles : sms * 4, TC_M, tc_smem(), s>>>(m->pack, m->P, X, n, out, m->err);
  counted();
  gfm_status_t r = ck(cudaGetLastError(), "k_mlp_infer_tc");
  int err = 0;
  if (r == GFM_OK) r = ck(cudaMemcpyAsync(&err, m->err, sizeof(int), cudaMemcpyDeviceToHost, s), "err");
  if (r == GFM_OK) r = ck(cudaStreamSynchronize(s), "infer");
  if (r == GFM_OK && err) r = GFM_ERR_CUDA;   // an mbarrier wait ran out
  return r;
}

gfm_status_t gfm_rs_mixed_batch_learned(gfm_mlp* m, int n, double gammaL, double pinfL, double gammaR, double pinfR,
                                        const double* UL, const double* UR, double* out, int* iters,
                                        uint32_t* status, int use_net, void* cuda_stream) {
  if (!m || n < 1 || !UL || !UR || !out || !iters || !status) return GFM_ERR_ARG;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(cuda_stream);
  if (use_net && m->pack_stale) {
    gfm_status_t r = repack(m, s);
    if (r != GFM_OK) return r;
  }
  cudaMemsetAsync(m->err, 0, sizeof(int), s);
  cudaFuncSetAttribute(k_rs_mixed_learned, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc_smem());
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int tiles = (n + TC_M - 1) / TC_M;
  k_rs_mixed_learned<<<tiles < sms * 4 ? tiles : sms * 4, TC_M, tc_smem(), s>>>(
      m->pack, m->P, n, make_gas(gammaL, pinfL), make_gas(gammaR, pinfR), UL, UR, out, iters, status, use_net ? 1 : 0,
      m->err);
  counted();
  gfm_status_t r = ck(cudaGetLastError(), "k_rs_mixed_learned");
  int err = 0;
  if (r == GFM_OK) r = ck(cudaMemcpyAsync(&err, m->err, sizeof(int), cudaMemcpyDeviceToHost, s), "err");
  if (r == GFM_OK) r = ck(cudaStreamSynchronize(s), "rs learned");
  if (r == GFM_OK && err) r = GFM_ERR_CUDA;
  return r;
}

}  // extern "C"
