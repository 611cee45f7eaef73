// FFT form of the contraction T = V Z of the matrix-free BSE operator on a two-dimensional Monkhorst-Pack mesh.
//
// The reference evaluates the screened potential at kpt(k) - kpt(k') element by element
// (src/module_bse.F90:49-72, matrizelbse).  On a mesh that difference depends on the index differences only,
// so V(k, k') = s(i - i', j - j') for k = (i, j), k' = (i', j') (coulomb_stencil_kernel builds s), and each
// column of T = V Z is the linear convolution of s ((2 n1 - 1) x (2 n2 - 1) values) with the column of Z laid
// out on the n1 x n2 mesh.  With a power of two P >= 2 max(n1, n2) - 1, the P x P cyclic convolution of the
// zero-padded column with s wrapped modulo P equals the linear one at the mesh points:
//   T = IDFT2(S o DFT2(z)) / P^2,   S = DFT2(s wrapped modulo P)   (S in FP64, stored in FP32 with 1 / P^2)
// s is real, so two real columns (the re and im rows n = 2q, 2q + 1 of one (b, o, p) item) go through one
// complex transform: the real part of the result is the first column's convolution, the imaginary part the
// second's.
//
// fft_conv_kernel: one CTA per complex column, 256 threads, FP32:
//   A. row transforms: DFT over j of the n1 nonzero rows of the padded grid (n2 nonzero inputs each) into a
//      shared n1 x P array;
//   B. column pass, for each of the P columns v: DFT over i (n1 nonzero inputs), times S(:, v), inverse DFT;
//      the n1 outputs on the mesh go back to the array;
//   C. inverse row transforms; the n2 outputs on the mesh are written to T (row k = i n2 + j, columns 2q, 2q + 1).
// A P-point transform is done by a group of G = P / 16 threads (Cooley-Tukey with P = G x 16): each thread a
// 16-point DFT over the stride-G subsequence r, r + G, ..., the twiddles W_P^(r k2), a transpose through the
// group's shared scratch, and 16 / G G-point DFTs.  Outputs are then "distributed": thread r holds
// X[k2 + 16 k1] for k2 = r (16 / G) + t, t < 16 / G, k1 < G, at x[t G + k1].  The inverse runs the same steps
// backwards from that layout, so the column pass needs no reordering.  At n1 = n2 = 60 (P = 128) a column
// takes 60 + 2 x 128 + 60 = 376 transforms of 128 points, about 1.7 MFLOP against the dense product's
// 2 x 3600^2 = 26 MFLOP per real column pair.
#include "wtb_internal.h"

#include <algorithm>

namespace wtb {
namespace {

__device__ __forceinline__ float2 c2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 cadd2(float2 a, float2 b) { return c2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub2(float2 a, float2 b) { return c2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul2(float2 a, float2 b) { return c2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
// a conj(b)
__device__ __forceinline__ float2 cmulc2(float2 a, float2 b) { return c2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y); }
__device__ __forceinline__ float2 conj2(float2 a) { return c2(a.x, -a.y); }
// -i a
__device__ __forceinline__ float2 mi2(float2 a) { return c2(a.y, -a.x); }

// W_16^k = exp(-2 pi i k / 16) for the twiddles inside a 16-point DFT: cos(pi / 8), sin(pi / 8), sqrt(1 / 2)
constexpr float kC1 = 0.923879532511286756f, kS1 = 0.382683432365089772f, kR = 0.707106781186547524f;

__device__ __forceinline__ void dft4(float2& a0, float2& a1, float2& a2, float2& a3) {
  const float2 t0 = cadd2(a0, a2), t1 = csub2(a0, a2), t2 = cadd2(a1, a3), t3 = csub2(a1, a3);
  a0 = cadd2(t0, t2);
  a2 = csub2(t0, t2);
  a1 = cadd2(t1, mi2(t3));
  a3 = csub2(t1, mi2(t3));
}

// X[k] = sum_m W_16^(m k) x[m], in place, as 4 x 4.  HALF: x[8..15] are zero (a zero-padded input), which
// halves the first stage.
template <bool HALF = false>
__device__ __forceinline__ void dft16(float2 (&x)[16]) {
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    if constexpr (HALF) {
      const float2 a0 = x[a], a1 = x[a + 4];
      x[a] = cadd2(a0, a1);
      x[a + 4] = cadd2(a0, mi2(a1));
      x[a + 8] = csub2(a0, a1);
      x[a + 12] = csub2(a0, mi2(a1));
    } else {
      dft4(x[a], x[a + 4], x[a + 8], x[a + 12]);
    }
  }
  // x[a + 4 c] now holds A[a][c] = sum_b W_4^(b c) x[a + 4 b]; twiddle by W_16^(a c)
  x[5] = cmul2(x[5], c2(kC1, -kS1));    // a 1, c 1
  x[9] = cmul2(x[9], c2(kR, -kR));      // a 1, c 2
  x[13] = cmul2(x[13], c2(kS1, -kC1));  // a 1, c 3
  x[6] = cmul2(x[6], c2(kR, -kR));      // a 2, c 1
  x[10] = mi2(x[10]);                   // a 2, c 2
  x[14] = cmul2(x[14], c2(-kR, -kR));   // a 2, c 3
  x[7] = cmul2(x[7], c2(kS1, -kC1));    // a 3, c 1
  x[11] = cmul2(x[11], c2(-kR, -kR));   // a 3, c 2
  x[15] = cmul2(x[15], c2(-kC1, kS1));  // a 3, c 3
  // X[c + 4 d] = sum_a W_4^(a d) A[a][c]
  float2 y[16];
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    float2 a0 = x[4 * c], a1 = x[4 * c + 1], a2 = x[4 * c + 2], a3 = x[4 * c + 3];
    dft4(a0, a1, a2, a3);
    y[c] = a0;
    y[c + 4] = a1;
    y[c + 8] = a2;
    y[c + 12] = a3;
  }
#pragma unroll
  for (int k = 0; k < 16; ++k) x[k] = y[k];
}

template <int G>
__device__ __forceinline__ void dftg(float2 (&z)[G]) {
  if constexpr (G == 2) {
    const float2 a = z[0], b = z[1];
    z[0] = cadd2(a, b);
    z[1] = csub2(a, b);
  } else if constexpr (G == 4) {
    dft4(z[0], z[1], z[2], z[3]);
  } else {
    static_assert(G == 8, "transform groups of 2, 4 or 8 threads");
    float2 e0 = z[0], e1 = z[2], e2 = z[4], e3 = z[6], o0 = z[1], o1 = z[3], o2 = z[5], o3 = z[7];
    dft4(e0, e1, e2, e3);
    dft4(o0, o1, o2, o3);
    o1 = cmul2(o1, c2(kR, -kR));
    o2 = mi2(o2);
    o3 = cmul2(o3, c2(-kR, -kR));
    z[0] = cadd2(e0, o0);
    z[4] = csub2(e0, o0);
    z[1] = cadd2(e1, o1);
    z[5] = csub2(e1, o1);
    z[2] = cadd2(e2, o2);
    z[6] = csub2(e2, o2);
    z[3] = cadd2(e3, o3);
    z[7] = csub2(e3, o3);
  }
}

// The twiddles W_P^(r k2), k2 < 16, of lane r: W^1, W^2, W^4, W^8 (W = W_P^r) are read once per thread from
// the FP64-rounded table; the others are products of at most three of them (a few ulp, below the transform's
// own log2(P) ulp), formed in registers so that the transforms issue no loads for them.
struct LaneTw {
  float2 w1, w2, w4, w8;
};

// x[k2] *= W^k2 (conj: times conj(W^k2)), k2 = 1..15
template <bool CONJ>
__device__ __forceinline__ void apply_tw(float2 (&x)[16], const LaneTw& t) {
  auto mul = [](float2 a, float2 w) { return CONJ ? cmulc2(a, w) : cmul2(a, w); };
  const float2 w3 = cmul2(t.w2, t.w1), w5 = cmul2(t.w4, t.w1), w6 = cmul2(t.w4, t.w2), w7 = cmul2(t.w4, w3);
  x[1] = mul(x[1], t.w1);
  x[2] = mul(x[2], t.w2);
  x[3] = mul(x[3], w3);
  x[4] = mul(x[4], t.w4);
  x[5] = mul(x[5], w5);
  x[6] = mul(x[6], w6);
  x[7] = mul(x[7], w7);
  x[8] = mul(x[8], t.w8);
  x[9] = mul(x[9], cmul2(t.w8, t.w1));
  x[10] = mul(x[10], cmul2(t.w8, t.w2));
  x[11] = mul(x[11], cmul2(t.w8, w3));
  x[12] = mul(x[12], cmul2(t.w8, t.w4));
  x[13] = mul(x[13], cmul2(t.w8, w5));
  x[14] = mul(x[14], cmul2(t.w8, w6));
  x[15] = mul(x[15], cmul2(t.w8, w7));
}

__device__ __forceinline__ void st2(float2* p, float2 a, float2 b) {
  *reinterpret_cast<float4*>(p) = make_float4(a.x, a.y, b.x, b.y);
}
__device__ __forceinline__ void ld2(const float2* p, float2& a, float2& b) {
  const float4 v = *reinterpret_cast<const float4*>(p);
  a = c2(v.x, v.y);
  b = c2(v.z, v.w);
}

// Scratch rows of 18 complex (16 used): 16-byte aligned pairs, and the 8 lanes of a group touch distinct banks.
constexpr int kScr = 18;

// P-point forward transform of a group of G = P / 16 threads (lane r of the group): on entry x[m] is element
// r + G m of the natural sequence; on return x[t G + k1] is X[k2 + 16 k1], k2 = r (16 / G) + t.  scr: the
// group's G x 18 scratch (16-byte aligned).  Every lane of the warp calls it (it synchronises the warp).
// HALF: the upper half of the sequence is zero (x[m] = 0 for m >= 8), as for a mesh row or column padded to P.
template <int P, bool HALF = false>
__device__ __forceinline__ void fft_fwd(float2 (&x)[16], int r, float2* scr, const LaneTw& tw) {
  constexpr int G = P / 16, T = 16 / G;
  dft16<HALF>(x);
  apply_tw<false>(x, tw);
  __syncwarp();  // the group's previous reads of the scratch are done
#pragma unroll
  for (int k2 = 0; k2 < 16; k2 += 2) st2(scr + r * kScr + k2, x[k2], x[k2 + 1]);
  __syncwarp();
  float2 z[T][G];
#pragma unroll
  for (int n1 = 0; n1 < G; ++n1)
#pragma unroll
    for (int t = 0; t < T; t += 2) ld2(scr + n1 * kScr + r * T + t, z[t][n1], z[t + 1][n1]);
#pragma unroll
  for (int t = 0; t < T; ++t) {
    dftg<G>(z[t]);
#pragma unroll
    for (int k1 = 0; k1 < G; ++k1) x[t * G + k1] = z[t][k1];
  }
}

// The unnormalised inverse of fft_fwd: from the distributed layout back to element r + G m at x[m].
template <int P>
__device__ __forceinline__ void fft_inv(float2 (&x)[16], int r, float2* scr, const LaneTw& tw) {
  constexpr int G = P / 16, T = 16 / G;
  float2 z[T][G];
#pragma unroll
  for (int t = 0; t < T; ++t) {
#pragma unroll
    for (int k1 = 0; k1 < G; ++k1) z[t][k1] = conj2(x[t * G + k1]);
    dftg<G>(z[t]);  // conj of the inverse G-point DFT
  }
  __syncwarp();
#pragma unroll
  for (int n1 = 0; n1 < G; ++n1)
#pragma unroll
    for (int t = 0; t < T; t += 2) st2(scr + n1 * kScr + r * T + t, conj2(z[t][n1]), conj2(z[t + 1][n1]));
  __syncwarp();
#pragma unroll
  for (int k2 = 0; k2 < 16; k2 += 2) ld2(scr + r * kScr + k2, x[k2], x[k2 + 1]);
  apply_tw<true>(x, tw);
#pragma unroll
  for (int k2 = 0; k2 < 16; ++k2) x[k2] = conj2(x[k2]);
  dft16(x);
#pragma unroll
  for (int k2 = 0; k2 < 16; ++k2) x[k2] = conj2(x[k2]);
}

constexpr int kFftThreads = 256;

// t_kn: T as [k][ldt] rows (column pair 2q, 2q + 1 of row k); otherwise T as [n][ldt] rows like Z.
// spec: the complex spectrum; spec_re its real parts (the same layout, FP32) and *even != 0 when the stencil is
// even, s(-d) = s(d) bitwise (every potential of the reference depends on q through |q| or squared components),
// so that the spectrum is real and the column pass multiplies by (and loads) its real parts only.
template <int P>
__global__ void __launch_bounds__(kFftThreads, 2) fft_conv_kernel(const float* __restrict__ Z, int ldz, int n1, int n2,
                                                                  const float2* __restrict__ spec,
                                                                  const float* __restrict__ spec_re,
                                                                  const int* __restrict__ even,
                                                                  const float2* __restrict__ tw_g,
                                                                  float* __restrict__ T, int ldt, int t_kn) {
  constexpr int G = P / 16, TT = 16 / G, NG = kFftThreads / G, LDS = P + 1, TS = 128 / P;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* scr_all = reinterpret_cast<float2*>(smem_raw);  // [NG][G * kScr]
  float2* Sb = scr_all + NG * G * kScr;                    // [n1][P + 1]
  const int tid = threadIdx.x, g = tid / G, r = tid % G;
  float2* scr = scr_all + g * (G * kScr);
  const int q = blockIdx.x;
  const float* zre = Z + (size_t)(2 * q) * ldz;
  const float* zim = zre + ldz;
  const LaneTw tw{tw_g[r * TS], tw_g[2 * r * TS], tw_g[4 * r * TS], tw_g[8 * r * TS]};
  const bool real_spec = *even != 0;  // uniform
  const float2 zero = c2(0.f, 0.f);
  // A. row transforms over j
  for (int i0 = 0; i0 < n1; i0 += NG) {
    const int i = i0 + g;
    const bool act = i < n1;
    float2 x[16];
#pragma unroll
    for (int m = 0; m < 8; ++m) {
      const int j = r + G * m;
      x[m] = (act && j < n2) ? c2(zre[i * n2 + j], zim[i * n2 + j]) : zero;
    }
#pragma unroll
    for (int m = 8; m < 16; ++m) x[m] = zero;
    fft_fwd<P, true>(x, r, scr, tw);  // n2 <= P / 2: elements m >= 8 of every lane are padding
    if (act) {
#pragma unroll
      for (int t = 0; t < TT; ++t)
#pragma unroll
        for (int k1 = 0; k1 < G; ++k1) Sb[i * LDS + r * TT + t + 16 * k1] = x[t * G + k1];
    }
  }
  __syncthreads();
  // B. column pass: transform over i, multiply by the stencil's spectrum, transform back
  for (int v0 = 0; v0 < P; v0 += NG) {
    const int v = v0 + g;
    const bool act = v < P;
    float2 x[16];
#pragma unroll
    for (int m = 0; m < 8; ++m) {
      const int i = r + G * m;
      x[m] = (act && i < n1) ? Sb[i * LDS + v] : zero;
    }
#pragma unroll
    for (int m = 8; m < 16; ++m) x[m] = zero;
    fft_fwd<P, true>(x, r, scr, tw);  // n1 <= P / 2
    if (act) {
      if (real_spec) {
        const float4* sv = reinterpret_cast<const float4*>(spec_re + (size_t)v * P + r * 16);
#pragma unroll
        for (int h = 0; h < 4; ++h) {
          const float4 s4 = sv[h];
          const float sr[4] = {s4.x, s4.y, s4.z, s4.w};
#pragma unroll
          for (int u = 0; u < 4; ++u) x[4 * h + u] = c2(x[4 * h + u].x * sr[u], x[4 * h + u].y * sr[u]);
        }
      } else {
        const float4* sv = reinterpret_cast<const float4*>(spec + (size_t)v * P + r * 16);
#pragma unroll
        for (int h = 0; h < 8; ++h) {
          const float4 s4 = sv[h];
          x[2 * h] = cmul2(x[2 * h], c2(s4.x, s4.y));
          x[2 * h + 1] = cmul2(x[2 * h + 1], c2(s4.z, s4.w));
        }
      }
    }
    fft_inv<P>(x, r, scr, tw);
    if (act) {
#pragma unroll
      for (int m = 0; m < 8; ++m) {  // rows i >= n1 (m >= 8 always) are padding
        const int i = r + G * m;
        if (i < n1) Sb[i * LDS + v] = x[m];
      }
    }
  }
  __syncthreads();
  // C. inverse row transforms (as conj(DFT(conj(.)))), the mesh's n2 outputs of each row to T
  for (int i0 = 0; i0 < n1; i0 += NG) {
    const int i = i0 + g;
    const bool act = i < n1;
    float2 x[16];
#pragma unroll
    for (int m = 0; m < 16; ++m) x[m] = act ? conj2(Sb[i * LDS + r + G * m]) : zero;
    fft_fwd<P>(x, r, scr, tw);
    if (act) {
      if (t_kn) {  // T[k][2q + (0, 1)]: one 8-byte (re, im) store per output
        float* tq = T + 2 * q;
#pragma unroll
        for (int t = 0; t < TT; ++t)
#pragma unroll
          for (int k1 = 0; k1 < G; ++k1) {
            const int j = r * TT + t + 16 * k1;
            if (j < n2) *reinterpret_cast<float2*>(tq + (size_t)(i * n2 + j) * ldt) = conj2(x[t * G + k1]);
          }
      } else {  // rows of Z's layout, T[2q][k] and T[2q + 1][k]: a lane's outputs j, j + 1 are adjacent
        float* tre = T + (size_t)(2 * q) * ldt + i * n2;
        float* tim = tre + ldt;
#pragma unroll
        for (int t = 0; t < TT; t += 2)
#pragma unroll
          for (int k1 = 0; k1 < G; ++k1) {
            const int j = r * TT + t + 16 * k1;  // even
            const float2 a = conj2(x[t * G + k1]), b = conj2(x[(t + 1) * G + k1]);
            if (((i * n2) & 1) == 0 && j + 1 < n2) {
              *reinterpret_cast<float2*>(tre + j) = c2(a.x, b.x);
              *reinterpret_cast<float2*>(tim + j) = c2(a.y, b.y);
            } else {
              if (j < n2) {
                tre[j] = a.x;
                tim[j] = a.y;
              }
              if (j + 1 < n2) {
                tre[j + 1] = b.x;
                tim[j + 1] = b.y;
              }
            }
          }
      }
    }
  }
}

// R[a][v] = sum_b s[a][b] W_P^(v (b - (n2 - 1))), a < 2 n1 - 1 (row transforms of the stencil, FP64; the
// twiddles W_P^m from a shared table, one sincospi per thread)
__global__ void spec_rows_kernel(const double* __restrict__ st, int n1, int n2, int P, zd* __restrict__ R) {
  __shared__ double wr[128], wi[128];
  const int a = blockIdx.x, v = threadIdx.x;
  if (v < P) {
    double sn, cs;
    sincospi(2.0 * v / P, &sn, &cs);
    wr[v] = cs;
    wi[v] = -sn;
  }
  __syncthreads();
  if (v >= P) return;
  const int s2 = 2 * n2 - 1;
  double re = 0.0, im = 0.0;
  int m = ((-v * (n2 - 1)) % P + P) % P;  // v (b - (n2 - 1)) mod P at b = 0, advanced by v per b
  for (int b = 0; b < s2; ++b) {
    const double x = st[(size_t)a * s2 + b];
    re += x * wr[m];
    im += x * wi[m];
    m += v;
    if (m >= P) m -= P;
  }
  R[(size_t)a * P + v] = mk<double>(re, im);
}

// S[u][v] = sum_a R[a][v] W_P^(u (a - (n1 - 1))) / P^2, stored in FP32 in the distributed layout of the
// column pass: column v's P values, value u = k2 + 16 k1 at v P + r 16 + t G + k1 with k2 = r (16 / G) + t
__global__ void spec_cols_kernel(const zd* __restrict__ R, int n1, int P, float2* __restrict__ spec,
                                 float* __restrict__ spec_re) {
  __shared__ double wr[128], wi[128];
  const int u = blockIdx.x, v = threadIdx.x;
  if (v < P) {
    double sn, cs;
    sincospi(2.0 * v / P, &sn, &cs);
    wr[v] = cs;
    wi[v] = -sn;
  }
  __syncthreads();
  if (v >= P) return;
  const int s1 = 2 * n1 - 1, G = P / 16, T = 16 / G;
  double re = 0.0, im = 0.0;
  int m = ((-u * (n1 - 1)) % P + P) % P;
  for (int a = 0; a < s1; ++a) {
    const zd x = R[(size_t)a * P + v];
    re += x.re * wr[m] - x.im * wi[m];
    im += x.im * wr[m] + x.re * wi[m];
    m += u;
    if (m >= P) m -= P;
  }
  const double sc = 1.0 / ((double)P * P);
  const int k2 = u % 16, k1 = u / 16, r = k2 / T, t = k2 % T;
  spec[(size_t)v * P + r * 16 + t * G + k1] = make_float2((float)(re * sc), (float)(im * sc));
  spec_re[(size_t)v * P + r * 16 + t * G + k1] = (float)(re * sc);
}

// *even = 1 when s[d] == s[-d] bitwise for every index difference d of the (2 n1 - 1) x (2 n2 - 1) stencil
__global__ void stencil_even_kernel(const double* __restrict__ st, int n1, int n2, int* __restrict__ even) {
  const int s1 = 2 * n1 - 1, s2 = 2 * n2 - 1, n = s1 * s2;
  int ok = 1;
  for (int e = threadIdx.x; e < n; e += blockDim.x) {
    const int a = e / s2, b = e - a * s2;
    ok &= st[e] == st[(size_t)(s1 - 1 - a) * s2 + (s2 - 1 - b)] ? 1 : 0;
  }
  ok = __syncthreads_and(ok);
  if (threadIdx.x == 0) *even = ok;
}

// the transforms' twiddles W_128^m, m < 128, rounded to FP32 from FP64
__global__ void twiddle_kernel(float2* __restrict__ tw) {
  const int m = threadIdx.x;
  if (m >= 128) return;
  double sn, cs;
  sincospi(2.0 * m / 128.0, &sn, &cs);
  tw[m] = make_float2((float)cs, (float)-sn);
}

template <int P>
size_t conv_smem(int n1) {
  return (size_t)(kFftThreads * kScr + n1 * (P + 1)) * sizeof(float2);
}

}  // namespace

int fft_conv_size(int n1, int n2) {
  const int m = std::max(n1, n2);
  if (n1 < 1 || n2 < 1) return 0;
  for (int P : {32, 64, 128})
    if (2 * m - 1 <= P) return P;
  return 0;
}

cudaError_t launch_fft_spectrum(const double* stencil, int n1, int n2, int P, zd* work, float2* spec, float2* tw,
                                cudaStream_t s) {
  if (P != 32 && P != 64 && P != 128) return cudaErrorInvalidValue;
  if (2 * n1 - 1 > P || 2 * n2 - 1 > P) return cudaErrorInvalidValue;
  float* spec_re = reinterpret_cast<float*>(spec + (size_t)P * P);
  int* even = reinterpret_cast<int*>(spec_re + (size_t)P * P);
  spec_rows_kernel<<<2 * n1 - 1, 128, 0, s>>>(stencil, n1, n2, P, work); ++g_launch_count;
  spec_cols_kernel<<<P, 128, 0, s>>>(work, n1, P, spec, spec_re); ++g_launch_count;
  stencil_even_kernel<<<1, 256, 0, s>>>(stencil, n1, n2, even); ++g_launch_count;
  twiddle_kernel<<<1, 128, 0, s>>>(tw); ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t launch_fft_conv(const float* Z, int ldz, int npairs, int n1, int n2, int P, const float2* spec,
                            const float2* tw, float* T, int ldt, bool t_kn, cudaStream_t s) {
  if (npairs < 1) return cudaSuccess;
  if (2 * n1 - 1 > P || 2 * n2 - 1 > P || (ldt & 1)) return cudaErrorInvalidValue;
  const int kn = t_kn ? 1 : 0;
  const float* spec_re = reinterpret_cast<const float*>(spec + (size_t)P * P);
  const int* even = reinterpret_cast<const int*>(spec_re + (size_t)P * P);
  switch (P) {
    case 32: {
      const size_t smem = conv_smem<32>(n1);
      cudaError_t e = raise_smem_limit(reinterpret_cast<const void*>(fft_conv_kernel<32>), smem);
      if (e != cudaSuccess) return e;
      fft_conv_kernel<32><<<npairs, kFftThreads, smem, s>>>(Z, ldz, n1, n2, spec, spec_re, even, tw, T, ldt, kn);
      break;
    }
    case 64: {
      const size_t smem = conv_smem<64>(n1);
      cudaError_t e = raise_smem_limit(reinterpret_cast<const void*>(fft_conv_kernel<64>), smem);
      if (e != cudaSuccess) return e;
      fft_conv_kernel<64><<<npairs, kFftThreads, smem, s>>>(Z, ldz, n1, n2, spec, spec_re, even, tw, T, ldt, kn);
      break;
    }
    case 128: {
      const size_t smem = conv_smem<128>(n1);
      cudaError_t e = raise_smem_limit(reinterpret_cast<const void*>(fft_conv_kernel<128>), smem);
      if (e != cudaSuccess) return e;
      fft_conv_kernel<128><<<npairs, kFftThreads, smem, s>>>(Z, ldz, n1, n2, spec, spec_re, even, tw, T, ldt, kn);
      break;
    }
    default:
      return cudaErrorInvalidValue;
  }
  ++g_launch_count;
  return cudaGetLastError();
}

}  // namespace wtb
