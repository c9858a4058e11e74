// In-repo Monte Carlo dose transport, one thread per decay history.
//
// Replaces MonteCarloCalculator (pyvoxeldosimetry/core/monte_carlo.py:10-172):
// decays sampled in proportion to the activity map (:44-50), isotropic
// emission (:52-58), beta energies from the nuclide's spectrum (the reference
// uses a constant placeholder, :60-64), transport and energy scoring
// (:66-102), dose rate per voxel (:104-137).  The reference never runs (its
// constructor raises, :38-40; cp.atomic.add does not exist, :78); the physics
// here is the builder's (stated in pyvoxeldosimetry_gb300/data/mc_physics.py):
// CSDA electrons with Highland multiple scattering on a voxel DDA, Woodcock-
// tracked photons with Klein-Nishina Compton (Kahn's sampling) and absorption.
//
// Determinism: every random number comes from Philox4x32-10 keyed by the seed
// and counted by (history, draw), energy is scored in unsigned 64-bit fixed
// point (2^-32 MeV) with integer atomics, and the floating point uses only
// IEEE +, -, *, / and sqrt (this file is compiled without FMA contraction) plus
// a logarithm written here from its atanh series.  A CPU implementation of the
// same algorithm therefore reproduces the energy grid bit for bit.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>

#include "pvd_common.cuh"

namespace pvd {
namespace mc {

constexpr int MAXG = 8;
constexpr float FIX_SCALE = 4294967296.0f;  // 2^32 per MeV
constexpr float ME = 0.51099895f;            // electron rest energy (MeV)
constexpr float X0W = 36.08f;                // radiation length of water (g/cm^2)
constexpr int MAX_E_STEPS = 100000;
constexpr int MAX_P_STEPS = 100000;

struct Tables {
  const float* beta_icdf;
  const float* range;
  const float* mu;
  const float* cfrac;
  int n_beta, n_range, n_ph;
  float range_de, ph_de;
  float gamma_e[MAXG], gamma_p[MAXG];
  int n_gamma;
  float beta_yield;
  float e_cut;
};

struct Geom {
  int n0, n1, n2;
  float v0, v1, v2;  // voxel size (cm) per axis
};

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void philox(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t lo0 = 0xD2511F53u * c[0], hi0 = __umulhi(0xD2511F53u, c[0]);
    const uint32_t lo1 = 0xCD9E8D57u * c[2], hi1 = __umulhi(0xCD9E8D57u, c[2]);
    const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0;
    c[1] = lo1;
    c[2] = n2;
    c[3] = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

struct Rng {
  uint32_t k0, k1, h0, h1, ctr;
  uint32_t buf[4];
  int used;
  __device__ void init(unsigned long long seed, unsigned long long hist) {
    k0 = (uint32_t)seed;
    k1 = (uint32_t)(seed >> 32);
    h0 = (uint32_t)hist;
    h1 = (uint32_t)(hist >> 32);
    ctr = 0;
    used = 4;
  }
  __device__ uint32_t next() {
    if (used == 4) {
      buf[0] = h0;
      buf[1] = h1;
      buf[2] = ctr++;
      buf[3] = 0x5EED0001u;
      philox(buf, k0, k1);
      used = 0;
    }
    return buf[used++];
  }
  // uniform in (0, 1]: 24 random bits, exact in float
  __device__ float u01() { return (float)((next() >> 8) + 1u) * (1.0f / 16777216.0f); }
};

// natural log for normal positive x: 2 atanh((m-1)/(m+1)) series on m in [1/sqrt2, sqrt2)
__device__ __forceinline__ float mc_log(float x) {
  int bits = __float_as_int(x);
  int e = ((bits >> 23) & 0xff) - 127;
  float m = __int_as_float((bits & 0x007fffff) | 0x3f800000);
  if (m > 1.41421356f) {
    m = m * 0.5f;
    e = e + 1;
  }
  const float z = (m - 1.0f) / (m + 1.0f);
  const float z2 = z * z;
  const float p = z * (2.0f + z2 * (0.666666667f + z2 * (0.4f + z2 * (0.285714286f + z2 * (0.222222222f + z2 * 0.181818182f)))));
  return p + (float)e * 0.693147181f;
}

__device__ __forceinline__ float lerp_table(const float* t, int n, float x_over_dx) {
  float xi = x_over_dx;
  if (!(xi >= 0.0f)) xi = 0.0f;  // also NaN
  if (xi > (float)(n - 1)) xi = (float)(n - 1);
  int i = (int)xi;
  if (i > n - 2) i = n - 2;
  const float f = xi - (float)i;
  return t[i] + f * (t[i + 1] - t[i]);
}

// kinetic energy with CSDA range R (inverse of the monotonic range table)
__device__ __forceinline__ float energy_of_range(const Tables& tb, float R) {
  const float* r = tb.range;
  if (R <= 0.0f) return 0.0f;
  int lo = 0, hi = tb.n_range - 1;
  if (R >= r[hi]) return (float)hi * tb.range_de;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (r[mid] <= R)
      lo = mid;
    else
      hi = mid;
  }
  const float f = (R - r[lo]) / (r[hi] - r[lo]);
  return ((float)lo + f) * tb.range_de;
}

__device__ __forceinline__ unsigned long long fix(float e) { return (unsigned long long)(e * FIX_SCALE); }

// deposits are summed per voxel in a register and flushed when the voxel changes
struct Scorer {
  unsigned long long* edep;
  long long cur;
  unsigned long long acc;
  __device__ void add(long long v, float e) {
    if (v != cur) {
      flush();
      cur = v;
    }
    acc += fix(e);
  }
  __device__ void flush() {
    if (cur >= 0 && acc) atomicAdd(edep + cur, acc);
    acc = 0;
  }
};

__device__ __forceinline__ void iso_dir(Rng& g, float& w0, float& w1, float& w2) {
  for (int it = 0; it < 64; ++it) {
    const float x1 = 2.0f * g.u01() - 1.0f, x2 = 2.0f * g.u01() - 1.0f;
    const float s = x1 * x1 + x2 * x2;
    if (s < 1.0f && s > 0.0f) {
      const float q = 2.0f * sqrtf(1.0f - s);
      w0 = x1 * q;
      w1 = x2 * q;
      w2 = 1.0f - 2.0f * s;
      return;
    }
  }
  w0 = 0.0f;
  w1 = 0.0f;
  w2 = 1.0f;
}

// orthonormal e1, e2 perpendicular to unit w
__device__ __forceinline__ void basis(float w0, float w1, float w2, float* e1, float* e2) {
  float a0 = 1.0f, a1 = 0.0f, a2 = 0.0f;
  if (w0 > 0.9f || w0 < -0.9f) {
    a0 = 0.0f;
    a1 = 1.0f;
  }
  const float d = a0 * w0 + a1 * w1 + a2 * w2;
  float b0 = a0 - d * w0, b1 = a1 - d * w1, b2 = a2 - d * w2;
  const float inv = 1.0f / sqrtf(b0 * b0 + b1 * b1 + b2 * b2);
  b0 = b0 * inv;
  b1 = b1 * inv;
  b2 = b2 * inv;
  e1[0] = b0;
  e1[1] = b1;
  e1[2] = b2;
  e2[0] = w1 * b2 - w2 * b1;
  e2[1] = w2 * b0 - w0 * b2;
  e2[2] = w0 * b1 - w1 * b0;
}

__device__ __forceinline__ void renorm(float& w0, float& w1, float& w2) {
  const float inv = 1.0f / sqrtf(w0 * w0 + w1 * w1 + w2 * w2);
  w0 = w0 * inv;
  w1 = w1 * inv;
  w2 = w2 * inv;
}

__device__ __forceinline__ bool inside(const Geom& G, int i0, int i1, int i2) {
  return i0 >= 0 && i0 < G.n0 && i1 >= 0 && i1 < G.n1 && i2 >= 0 && i2 < G.n2;
}

__device__ __forceinline__ float density_at(const float* rho, const Geom& G, int i0, int i1, int i2) {
  if (!rho) return 1.0f;
  const float d = rho[((long long)i0 * G.n1 + i1) * G.n2 + i2];
  return (d > 1e-6f) ? d : 1e-6f;  // NaN / non-positive -> near vacuum
}

// ---------------------------------------------------------------------------
// electron: CSDA steps on the voxel grid, Highland multiple scattering
// ---------------------------------------------------------------------------
__device__ void transport_electron(const Tables& tb, const Geom& G, const float* rho, Rng& g, Scorer& sc, float E,
                                   float p0, float p1, float p2, int i0, int i1, int i2, float w0, float w1, float w2,
                                   unsigned long long& escaped, unsigned long long& steps) {
  float R = lerp_table(tb.range, tb.n_range, E / tb.range_de);
  for (int it = 0; it < MAX_E_STEPS && E > tb.e_cut; ++it) {
    ++steps;
    const long long v = ((long long)i0 * G.n1 + i1) * G.n2 + i2;
    const float d = density_at(rho, G, i0, i1, i2);
    // distance to the next voxel face (index-based faces: no zero-length loops)
    float db = 3.0e38f;
    int ax = -1;
    if (w0 > 0.0f) { const float t = ((float)(i0 + 1) * G.v0 - p0) / w0; if (t < db) { db = t; ax = 0; } }
    if (w0 < 0.0f) { const float t = ((float)i0 * G.v0 - p0) / w0; if (t < db) { db = t; ax = 0; } }
    if (w1 > 0.0f) { const float t = ((float)(i1 + 1) * G.v1 - p1) / w1; if (t < db) { db = t; ax = 1; } }
    if (w1 < 0.0f) { const float t = ((float)i1 * G.v1 - p1) / w1; if (t < db) { db = t; ax = 1; } }
    if (w2 > 0.0f) { const float t = ((float)(i2 + 1) * G.v2 - p2) / w2; if (t < db) { db = t; ax = 2; } }
    if (w2 < 0.0f) { const float t = ((float)i2 * G.v2 - p2) / w2; if (t < db) { db = t; ax = 2; } }
    if (db < 0.0f) db = 0.0f;
    const float smax = 0.25f * R / d;
    const bool cross = db <= smax;
    const float s = cross ? db : smax;
    const float t = d * s;
    if (t >= R) {  // stops inside this step
      sc.add(v, E);
      E = 0.0f;
      break;
    }
    const float Rn = R - t;
    const float En = energy_of_range(tb, Rn);
    if (E > En) sc.add(v, E - En);
    p0 = p0 + s * w0;
    p1 = p1 + s * w1;
    p2 = p2 + s * w2;
    if (cross) {
      if (ax == 0) i0 += (w0 > 0.0f) ? 1 : -1;
      if (ax == 1) i1 += (w1 > 0.0f) ? 1 : -1;
      if (ax == 2) i2 += (w2 > 0.0f) ? 1 : -1;
      if (!inside(G, i0, i1, i2)) {
        escaped += fix(En);
        E = 0.0f;
        break;
      }
    }
    // Highland width for the step's mass thickness at the mean step energy
    const float x = t / X0W;
    if (x > 1e-6f) {
      const float Em = 0.5f * (E + En);
      const float bcp = Em * (Em + 2.0f * ME) / (Em + ME);
      float fac = 1.0f + 0.038f * mc_log(x);
      if (fac < 0.0f) fac = 0.0f;
      const float th0 = 13.6f / bcp * sqrtf(x) * fac;
      if (th0 > 0.0f) {
        float g1 = 0.0f, g2 = 0.0f;
        for (int k = 0; k < 64; ++k) {  // Marsaglia polar Gaussian pair
          const float a = 2.0f * g.u01() - 1.0f, b = 2.0f * g.u01() - 1.0f;
          const float q = a * a + b * b;
          if (q < 1.0f && q > 0.0f) {
            const float f = sqrtf(-2.0f * mc_log(q) / q);
            g1 = a * f;
            g2 = b * f;
            break;
          }
        }
        float e1[3], e2[3];
        basis(w0, w1, w2, e1, e2);
        w0 = w0 + th0 * (g1 * e1[0] + g2 * e2[0]);
        w1 = w1 + th0 * (g1 * e1[1] + g2 * e2[1]);
        w2 = w2 + th0 * (g1 * e1[2] + g2 * e2[2]);
        renorm(w0, w1, w2);
      }
    }
    E = En;
    R = Rn;
  }
  if (E > 0.0f) sc.add(((long long)i0 * G.n1 + i1) * G.n2 + i2, E);
}

// ---------------------------------------------------------------------------
// photon: Woodcock tracking, absorption or Klein-Nishina Compton (local electron)
// ---------------------------------------------------------------------------
__device__ void transport_photon(const Tables& tb, const Geom& G, const float* rho, float rho_max, Rng& g, Scorer& sc,
                                 float E, float p0, float p1, float p2, int i0, int i1, int i2, float w0, float w1,
                                 float w2, unsigned long long& escaped, unsigned long long& steps) {
  for (int it = 0; it < MAX_P_STEPS; ++it) {
    ++steps;
    if (E <= tb.e_cut) {
      sc.add(((long long)i0 * G.n1 + i1) * G.n2 + i2, E);
      return;
    }
    const float mu = lerp_table(tb.mu, tb.n_ph, E / tb.ph_de);
    const float s = -mc_log(g.u01()) / (mu * rho_max);
    p0 = p0 + s * w0;
    p1 = p1 + s * w1;
    p2 = p2 + s * w2;
    const float f0 = p0 / G.v0, f1 = p1 / G.v1, f2 = p2 / G.v2;
    if (f0 < 0.0f || f1 < 0.0f || f2 < 0.0f || f0 >= (float)G.n0 || f1 >= (float)G.n1 || f2 >= (float)G.n2) {
      escaped += fix(E);
      return;
    }
    i0 = (int)f0;
    i1 = (int)f1;
    i2 = (int)f2;
    if (i0 >= G.n0) i0 = G.n0 - 1;
    if (i1 >= G.n1) i1 = G.n1 - 1;
    if (i2 >= G.n2) i2 = G.n2 - 1;
    const float d = density_at(rho, G, i0, i1, i2);
    if (g.u01() * rho_max > d) continue;  // virtual interaction
    const long long v = ((long long)i0 * G.n1 + i1) * G.n2 + i2;
    const float cf = lerp_table(tb.cfrac, tb.n_ph, E / tb.ph_de);
    if (g.u01() > cf) {  // absorption
      sc.add(v, E);
      return;
    }
    // Compton: Kahn's rejection sampling of eta = E / E'
    const float k = E / ME;
    float eta = 1.0f;
    for (int r = 0; r < 1000; ++r) {
      const float r1 = g.u01(), r2 = g.u01(), r3 = g.u01();
      if (r1 <= (1.0f + 2.0f * k) / (9.0f + 2.0f * k)) {
        const float et = 1.0f + 2.0f * k * r2;
        if (r3 <= 4.0f * (1.0f / et - 1.0f / (et * et))) {
          eta = et;
          break;
        }
      } else {
        const float et = (1.0f + 2.0f * k) / (1.0f + 2.0f * k * r2);
        const float ct = 1.0f - (et - 1.0f) / k;
        if (r3 <= 0.5f * (ct * ct + 1.0f / et)) {
          eta = et;
          break;
        }
      }
    }
    const float En = E / eta;
    float ct = 1.0f - (eta - 1.0f) / k;
    if (ct > 1.0f) ct = 1.0f;
    if (ct < -1.0f) ct = -1.0f;
    sc.add(v, E - En);
    const float st = sqrtf(1.0f - ct * ct);
    float c1 = 1.0f, s1 = 0.0f;
    for (int r = 0; r < 64; ++r) {  // uniform azimuth from a point of the unit disk
      const float a = 2.0f * g.u01() - 1.0f, b = 2.0f * g.u01() - 1.0f;
      const float q = a * a + b * b;
      if (q < 1.0f && q > 0.0f) {
        const float inv = 1.0f / sqrtf(q);
        c1 = a * inv;
        s1 = b * inv;
        break;
      }
    }
    float e1[3], e2[3];
    basis(w0, w1, w2, e1, e2);
    w0 = ct * w0 + st * (c1 * e1[0] + s1 * e2[0]);
    w1 = ct * w1 + st * (c1 * e1[1] + s1 * e2[1]);
    w2 = ct * w2 + st * (c1 * e1[2] + s1 * e2[2]);
    renorm(w0, w1, w2);
    E = En;
  }
}

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------
// max of activity (>= 0, NaN -> 0) and of density, as float bit patterns (order preserving)
__global__ void k_maxes(const float* __restrict__ act, const float* __restrict__ rho, long long n,
                        unsigned int* __restrict__ out) {
  unsigned int ma = 0, mr = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float a = act[i];
    if (a > 0.0f) ma = max(ma, __float_as_uint(a));
    if (rho) {
      const float d = rho[i];
      if (d > 0.0f) mr = max(mr, __float_as_uint(d));
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    ma = max(ma, __shfl_xor_sync(0xffffffffu, ma, o));
    mr = max(mr, __shfl_xor_sync(0xffffffffu, mr, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(out, ma);
    atomicMax(out + 1, mr);
  }
}

constexpr int SCAN_BLOCK = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_BLOCK * SCAN_ITEMS;

// w_i = (u64)(max(a_i, 0) * (2^32 / a_max)); per-tile inclusive prefix + tile totals
__global__ void __launch_bounds__(SCAN_BLOCK) k_weights_scan(const float* __restrict__ act, long long n,
                                                             const unsigned int* __restrict__ maxes,
                                                             unsigned long long* __restrict__ prefix,
                                                             unsigned long long* __restrict__ tile_sum) {
  __shared__ unsigned long long warp_tot[SCAN_BLOCK / 32];
  const float amax = __uint_as_float(maxes[0]);
  const float scale = (amax > 0.0f) ? FIX_SCALE / amax : 0.0f;
  const long long base = (long long)blockIdx.x * SCAN_TILE + (long long)threadIdx.x * SCAN_ITEMS;
  unsigned long long w[SCAN_ITEMS];
  unsigned long long run = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    const long long i = base + k;
    float a = (i < n) ? act[i] : 0.0f;
    if (!(a > 0.0f)) a = 0.0f;
    run += (unsigned long long)(a * scale);
    w[k] = run;
  }
  // warp inclusive scan of the per-thread totals
  unsigned long long x = run;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[wid] = x;
  __syncthreads();
  if (wid == 0) {
    unsigned long long t = (lane < SCAN_BLOCK / 32) ? warp_tot[lane] : 0ull;
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    if (lane < SCAN_BLOCK / 32) warp_tot[lane] = t;
  }
  __syncthreads();
  const unsigned long long excl = x - run + (wid > 0 ? warp_tot[wid - 1] : 0ull);
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    const long long i = base + k;
    if (i < n) prefix[i] = w[k] + excl;
  }
  if (threadIdx.x == SCAN_BLOCK - 1) tile_sum[blockIdx.x] = excl + run;
}

// exclusive scan of the tile totals (one block, sequential chunks)
__global__ void k_scan_tiles(unsigned long long* __restrict__ tile_sum, long long ntiles,
                             unsigned long long* __restrict__ total) {
  __shared__ unsigned long long carry;
  __shared__ unsigned long long warp_tot[32];
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (long long c0 = 0; c0 < ntiles; c0 += blockDim.x) {
    const long long i = c0 + threadIdx.x;
    const unsigned long long v = (i < ntiles) ? tile_sum[i] : 0ull;
    unsigned long long x = v;
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[wid] = x;
    __syncthreads();
    if (wid == 0) {
      unsigned long long t = (lane < (int)(blockDim.x / 32)) ? warp_tot[lane] : 0ull;
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, t, o);
        if (lane >= o) t += y;
      }
      warp_tot[lane] = t;
    }
    __syncthreads();
    const unsigned long long excl = carry + x - v + (wid > 0 ? warp_tot[wid - 1] : 0ull);
    if (i < ntiles) tile_sum[i] = excl;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = excl + v;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

__global__ void k_add_tile_offsets(unsigned long long* __restrict__ prefix, long long n,
                                   const unsigned long long* __restrict__ tile_off) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    prefix[i] += tile_off[i / SCAN_TILE];
}

__global__ void k_transport(Tables tb, Geom G, const float* __restrict__ rho, const unsigned int* __restrict__ maxes,
                            const unsigned long long* __restrict__ prefix, const unsigned long long* __restrict__ total,
                            unsigned long long n_hist, unsigned long long seed, unsigned long long* __restrict__ edep,
                            unsigned long long* __restrict__ counters) {
  const unsigned long long tot = *total;
  if (tot == 0) return;
  const float rho_max = rho ? __uint_as_float(maxes[1]) : 1.0f;
  const long long nvox = (long long)G.n0 * G.n1 * G.n2;
  unsigned long long emitted = 0, escaped = 0, steps = 0;
  Scorer sc{edep, -1, 0};
  for (unsigned long long h = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; h < n_hist;
       h += (unsigned long long)gridDim.x * blockDim.x) {
    Rng g;
    g.init(seed, h);
    // source voxel: first prefix entry above a uniform integer in [0, total)
    const unsigned long long rhi = g.next();  // two statements: the draw order is fixed
    const unsigned long long r = (rhi << 32) | g.next();
    const unsigned long long target = __umul64hi(r, tot);
    long long lo = 0, hi = nvox - 1;
    while (lo < hi) {
      const long long mid = (lo + hi) >> 1;
      if (prefix[mid] > target)
        hi = mid;
      else
        lo = mid + 1;
    }
    const int i2 = (int)(lo % G.n2), i1 = (int)((lo / G.n2) % G.n1), i0 = (int)(lo / ((long long)G.n1 * G.n2));
    const float p0 = ((float)i0 + g.u01()) * G.v0, p1 = ((float)i1 + g.u01()) * G.v1,
                p2 = ((float)i2 + g.u01()) * G.v2;
    if (tb.beta_yield > 0.0f && g.u01() <= tb.beta_yield) {
      const float E = lerp_table(tb.beta_icdf, tb.n_beta, g.u01() * (float)(tb.n_beta - 1));
      emitted += fix(E);
      float w0, w1, w2;
      iso_dir(g, w0, w1, w2);
      transport_electron(tb, G, rho, g, sc, E, p0, p1, p2, i0, i1, i2, w0, w1, w2, escaped, steps);
    }
    for (int l = 0; l < tb.n_gamma; ++l) {
      if (g.u01() <= tb.gamma_p[l]) {
        const float E = tb.gamma_e[l];
        emitted += fix(E);
        float w0, w1, w2;
        iso_dir(g, w0, w1, w2);
        transport_photon(tb, G, rho, rho_max, g, sc, E, p0, p1, p2, i0, i1, i2, w0, w1, w2, escaped, steps);
      }
    }
  }
  sc.flush();
  atomicAdd(counters + 0, emitted);
  atomicAdd(counters + 1, escaped);
  atomicAdd(counters + 2, steps);
}

// dose rate (Gy/s) = E[MeV] * (activity represented per history) * J/MeV / voxel mass; FP64 normalisation
__global__ void k_dose(const unsigned long long* __restrict__ edep, const float* __restrict__ rho, long long n,
                       const unsigned int* __restrict__ maxes, const unsigned long long* __restrict__ total,
                       unsigned long long n_hist, double voxel_cm3, float* __restrict__ dose) {
  const float amax = __uint_as_float(maxes[0]);
  const double scale = (amax > 0.0f) ? (double)(FIX_SCALE / amax) : 0.0;
  const double bq = (scale > 0.0) ? (double)(*total) / scale : 0.0;
  const double f = (n_hist > 0) ? bq / (double)n_hist * 1.602176634e-13 / 4294967296.0 / (voxel_cm3 * 1e-3) : 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double d = rho ? (double)rho[i] : 1.0;
    dose[i] = (d > 0.0) ? (float)((double)edep[i] * f / d) : 0.0f;
  }
}

}  // namespace mc
}  // namespace pvd

using namespace pvd;
using namespace pvd::mc;

struct pvd_mc_plan {
  Tables tb;
  Geom G;
  double voxel_cm3;
  long long nvox = 0;
  long long ntiles = 0;
  float* d_tables = nullptr;               // beta | range | mu | cfrac
  unsigned long long* d_prefix = nullptr;  // nvox
  unsigned long long* d_tiles = nullptr;   // ntiles
  unsigned long long* d_misc = nullptr;    // [0] total weight, [1..4] counters
  unsigned int* d_max = nullptr;           // [0] activity max bits, [1] density max bits
};

extern "C" pvd_status pvd_mc_plan_create(const pvd_mc_desc* d, pvd_mc_plan** out) {
  if (!d || !out) return set_error(PVD_ERR_ARG, "pvd_mc_plan_create: null argument");
  *out = nullptr;
  for (int i = 0; i < 3; ++i) {
    if (d->n[i] < 1 || d->n[i] > 4096) return set_error(PVD_ERR_ARG, "pvd_mc_plan_create: dims must be in [1, 4096]");
    if (!(d->voxel_mm[i] > 0.0)) return set_error(PVD_ERR_ARG, "pvd_mc_plan_create: voxel size must be > 0");
  }
  if (!d->beta_icdf || d->n_beta < 2 || !d->range || d->n_range < 2 || !(d->range_de > 0.0f) || !d->mu_rho ||
      !d->compton_frac || d->n_photon < 2 || !(d->photon_de > 0.0f))
    return set_error(PVD_ERR_ARG, "pvd_mc_plan_create: physics tables missing or too short");
  if (d->n_gamma < 0 || d->n_gamma > PVD_MC_MAX_GAMMA) return set_error(PVD_ERR_ARG, "pvd_mc_plan_create: n_gamma out of range");
  for (int l = 0; l < d->n_gamma; ++l)
    if (!(d->gamma_e[l] > 0.0f) || (float)((d->n_photon - 1)) * d->photon_de < d->gamma_e[l])
      return set_error(PVD_ERR_ARG, "pvd_mc_plan_create: gamma line outside the photon tables");
  if ((float)(d->n_range - 1) * d->range_de < d->beta_icdf[d->n_beta - 1])
    return set_error(PVD_ERR_ARG, "pvd_mc_plan_create: beta end point outside the range table");
  pvd_mc_plan* p = new pvd_mc_plan();
  p->G.n0 = d->n[0];
  p->G.n1 = d->n[1];
  p->G.n2 = d->n[2];
  p->G.v0 = (float)(d->voxel_mm[0] * 0.1);
  p->G.v1 = (float)(d->voxel_mm[1] * 0.1);
  p->G.v2 = (float)(d->voxel_mm[2] * 0.1);
  p->voxel_cm3 = d->voxel_mm[0] * d->voxel_mm[1] * d->voxel_mm[2] * 1e-3;
  p->nvox = (long long)d->n[0] * d->n[1] * d->n[2];
  p->ntiles = (p->nvox + SCAN_TILE - 1) / SCAN_TILE;
  const size_t nt = (size_t)d->n_beta + d->n_range + 2 * (size_t)d->n_photon;
  cudaError_t e = cudaMalloc(&p->d_tables, sizeof(float) * nt);
  if (e == cudaSuccess) e = cudaMalloc(&p->d_prefix, sizeof(unsigned long long) * p->nvox);
  if (e == cudaSuccess) e = cudaMalloc(&p->d_tiles, sizeof(unsigned long long) * p->ntiles);
  if (e == cudaSuccess) e = cudaMalloc(&p->d_misc, sizeof(unsigned long long) * 8);
  if (e == cudaSuccess) e = cudaMalloc(&p->d_max, sizeof(unsigned int) * 2);
  float* t = p->d_tables;
  if (e == cudaSuccess) e = cudaMemcpy(t, d->beta_icdf, sizeof(float) * d->n_beta, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(t + d->n_beta, d->range, sizeof(float) * d->n_range, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(t + d->n_beta + d->n_range, d->mu_rho, sizeof(float) * d->n_photon, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(t + d->n_beta + d->n_range + d->n_photon, d->compton_frac, sizeof(float) * d->n_photon,
                   cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaGetLastError();
    cudaFree(p->d_tables);
    cudaFree(p->d_prefix);
    cudaFree(p->d_tiles);
    cudaFree(p->d_misc);
    cudaFree(p->d_max);
    delete p;
    return cuda_error(e, "pvd_mc_plan_create");
  }
  Tables& tb = p->tb;
  tb.beta_icdf = t;
  tb.range = t + d->n_beta;
  tb.mu = t + d->n_beta + d->n_range;
  tb.cfrac = t + d->n_beta + d->n_range + d->n_photon;
  tb.n_beta = d->n_beta;
  tb.n_range = d->n_range;
  tb.n_ph = d->n_photon;
  tb.range_de = d->range_de;
  tb.ph_de = d->photon_de;
  tb.n_gamma = d->n_gamma;
  for (int l = 0; l < MAXG; ++l) {
    tb.gamma_e[l] = l < d->n_gamma ? d->gamma_e[l] : 0.0f;
    tb.gamma_p[l] = l < d->n_gamma ? d->gamma_yield[l] : 0.0f;
  }
  tb.beta_yield = d->beta_yield;
  tb.e_cut = d->e_cut;
  *out = p;
  return PVD_OK;
}

extern "C" pvd_status pvd_mc_run(pvd_mc_plan* p, const float* activity_d, const float* density_d,
                                 unsigned long long n_histories, unsigned long long seed, unsigned long long* edep_d,
                                 float* dose_rate_d, pvd_mc_stats* stats, pvd_stream stream) {
  if (!p || !activity_d || !edep_d) return set_error(PVD_ERR_ARG, "pvd_mc_run: null argument");
  cudaStream_t st = (cudaStream_t)stream;
  const long long n = p->nvox;
  PVD_CUDA_TRY(cudaMemsetAsync(edep_d, 0, sizeof(unsigned long long) * n, st));
  PVD_CUDA_TRY(cudaMemsetAsync(p->d_misc, 0, sizeof(unsigned long long) * 8, st));
  PVD_CUDA_TRY(cudaMemsetAsync(p->d_max, 0, sizeof(unsigned int) * 2, st));
  const int gs = 152 * 8;
  k_maxes<<<gs, 256, 0, st>>>(activity_d, density_d, n, p->d_max);
  PVD_LAUNCH_CHECK("k_maxes");
  k_weights_scan<<<(unsigned)p->ntiles, SCAN_BLOCK, 0, st>>>(activity_d, n, p->d_max, p->d_prefix, p->d_tiles);
  PVD_LAUNCH_CHECK("k_weights_scan");
  k_scan_tiles<<<1, 1024, 0, st>>>(p->d_tiles, p->ntiles, p->d_misc);
  PVD_LAUNCH_CHECK("k_scan_tiles");
  k_add_tile_offsets<<<gs, 256, 0, st>>>(p->d_prefix, n, p->d_tiles);
  PVD_LAUNCH_CHECK("k_add_tile_offsets");
  if (n_histories > 0) {
    const unsigned long long want = (n_histories + 127) / 128;
    const int blocks = (int)std::min<unsigned long long>(want, 152ull * 64);
    k_transport<<<blocks, 128, 0, st>>>(p->tb, p->G, density_d, p->d_max, p->d_prefix, p->d_misc, n_histories, seed,
                                         edep_d, p->d_misc + 1);
    PVD_LAUNCH_CHECK("k_transport");
  }
  if (dose_rate_d) {
    k_dose<<<gs, 256, 0, st>>>(edep_d, density_d, n, p->d_max, p->d_misc, n_histories, p->voxel_cm3, dose_rate_d);
    PVD_LAUNCH_CHECK("k_dose");
  }
  if (stats) {
    unsigned long long h[4];
    unsigned int m[2];
    PVD_CUDA_TRY(cudaMemcpyAsync(h, p->d_misc, sizeof(h), cudaMemcpyDeviceToHost, st));
    PVD_CUDA_TRY(cudaMemcpyAsync(m, p->d_max, sizeof(m), cudaMemcpyDeviceToHost, st));
    PVD_CUDA_TRY(cudaStreamSynchronize(st));
    float amax;
    std::memcpy(&amax, &m[0], sizeof(float));
    const double scale = amax > 0.0f ? (double)(FIX_SCALE / amax) : 0.0;
    stats->total_weight = h[0];
    stats->emitted = h[1];
    stats->escaped = h[2];
    stats->steps = h[3];
    stats->activity_bq = scale > 0.0 ? (double)h[0] / scale : 0.0;
  }
  return PVD_OK;
}

extern "C" pvd_status pvd_mc_plan_destroy(pvd_mc_plan* p) {
  if (!p) return PVD_OK;
  cudaFree(p->d_tables);
  cudaFree(p->d_prefix);
  cudaFree(p->d_tiles);
  cudaFree(p->d_misc);
  cudaFree(p->d_max);
  delete p;
  return PVD_OK;
}
