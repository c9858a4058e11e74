/*
 * ORACLE — test infrastructure only, never the product path.
 *
 * Plain-C restatement of the in-repo Monte Carlo dose transport, one history
 * after another on the CPU.  The reference's MonteCarloCalculator
 * (pyvoxeldosimetry/core/monte_carlo.py:10-172) cannot run (its constructor
 * raises at :38-40), so the MC is "parity unpinned" against the reference
 * itself; this oracle restates the builder's algorithm independently so the
 * GPU result can be checked bit for bit: the same Philox4x32-10 streams
 * (Salmon et al., SC'11), the same IEEE single-precision operation sequence
 * (compile with -ffp-contract=off, no fast-math), the same atanh-series
 * logarithm, and energy scored in unsigned 64-bit fixed point (2^-32 MeV).
 *
 * Build: see oracle/__init__.py (gcc -O2 -ffp-contract=off -fPIC -shared).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define FIXS 4294967296.0f
#define MEC2 0.51099895f
#define X0WATER 36.08f

typedef struct {
  const float *beta, *range, *mu, *cf;
  int nb, nr, np;
  float rde, pde;
  int ng;
  const float *ge, *gp;
  float by, ecut;
  int n0, n1, n2;
  float v0, v1, v2;
  const float* rho;
  float rho_max;
} world;

typedef struct {
  uint32_t k0, k1, h0, h1, c;
  uint32_t b[4];
  int u;
} stream;

static uint32_t hi32(uint32_t a, uint32_t b) { return (uint32_t)(((uint64_t)a * (uint64_t)b) >> 32); }

static void philox10(uint32_t x[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    uint32_t a0 = x[0], a2 = x[2];
    uint32_t p0lo = 0xD2511F53u * a0, p0hi = hi32(0xD2511F53u, a0);
    uint32_t p1lo = 0xCD9E8D57u * a2, p1hi = hi32(0xCD9E8D57u, a2);
    uint32_t y0 = p1hi ^ x[1] ^ k0;
    uint32_t y2 = p0hi ^ x[3] ^ k1;
    x[0] = y0;
    x[1] = p1lo;
    x[2] = y2;
    x[3] = p0lo;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

static uint32_t draw(stream* s) {
  if (s->u == 4) {
    s->b[0] = s->h0;
    s->b[1] = s->h1;
    s->b[2] = s->c++;
    s->b[3] = 0x5EED0001u;
    philox10(s->b, s->k0, s->k1);
    s->u = 0;
  }
  return s->b[s->u++];
}

static float unif(stream* s) { return (float)((draw(s) >> 8) + 1u) * (1.0f / 16777216.0f); }

/* ln x = 2 atanh((m-1)/(m+1)) + e ln 2, m in [1/sqrt2, sqrt2) */
static float ln_f(float x) {
  int32_t bits;
  memcpy(&bits, &x, 4);
  int e = ((bits >> 23) & 0xff) - 127;
  int32_t mb = (bits & 0x007fffff) | 0x3f800000;
  float m;
  memcpy(&m, &mb, 4);
  if (m > 1.41421356f) {
    m = m * 0.5f;
    e = e + 1;
  }
  float z = (m - 1.0f) / (m + 1.0f);
  float z2 = z * z;
  float poly = z * (2.0f + z2 * (0.666666667f + z2 * (0.4f + z2 * (0.285714286f + z2 * (0.222222222f + z2 * 0.181818182f)))));
  return poly + (float)e * 0.693147181f;
}

static float interp(const float* t, int n, float xdx) {
  float x = xdx;
  if (!(x >= 0.0f)) x = 0.0f;
  if (x > (float)(n - 1)) x = (float)(n - 1);
  int i = (int)x;
  if (i > n - 2) i = n - 2;
  float f = x - (float)i;
  return t[i] + f * (t[i + 1] - t[i]);
}

static float e_of_r(const world* w, float R) {
  if (R <= 0.0f) return 0.0f;
  int lo = 0, hi = w->nr - 1;
  if (R >= w->range[hi]) return (float)hi * w->rde;
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (w->range[mid] <= R)
      lo = mid;
    else
      hi = mid;
  }
  float f = (R - w->range[lo]) / (w->range[hi] - w->range[lo]);
  return ((float)lo + f) * w->rde;
}

static uint64_t q32(float e) { return (uint64_t)(e * FIXS); }

static float rho_at(const world* w, int a, int b, int c) {
  if (!w->rho) return 1.0f;
  float d = w->rho[((int64_t)a * w->n1 + b) * w->n2 + c];
  return (d > 1e-6f) ? d : 1e-6f;
}

static int64_t vox(const world* w, int a, int b, int c) { return ((int64_t)a * w->n1 + b) * w->n2 + c; }

static void direction(stream* s, float* d) {
  for (int it = 0; it < 64; ++it) {
    float x1 = 2.0f * unif(s) - 1.0f, x2 = 2.0f * unif(s) - 1.0f;
    float q = x1 * x1 + x2 * x2;
    if (q < 1.0f && q > 0.0f) {
      float f = 2.0f * sqrtf(1.0f - q);
      d[0] = x1 * f;
      d[1] = x2 * f;
      d[2] = 1.0f - 2.0f * q;
      return;
    }
  }
  d[0] = 0.0f;
  d[1] = 0.0f;
  d[2] = 1.0f;
}

static void perp(const float* d, float* e1, float* e2) {
  float a0 = 1.0f, a1 = 0.0f, a2 = 0.0f;
  if (d[0] > 0.9f || d[0] < -0.9f) {
    a0 = 0.0f;
    a1 = 1.0f;
  }
  float dot = a0 * d[0] + a1 * d[1] + a2 * d[2];
  float b0 = a0 - dot * d[0], b1 = a1 - dot * d[1], b2 = a2 - dot * d[2];
  float inv = 1.0f / sqrtf(b0 * b0 + b1 * b1 + b2 * b2);
  b0 = b0 * inv;
  b1 = b1 * inv;
  b2 = b2 * inv;
  e1[0] = b0;
  e1[1] = b1;
  e1[2] = b2;
  e2[0] = d[1] * b2 - d[2] * b1;
  e2[1] = d[2] * b0 - d[0] * b2;
  e2[2] = d[0] * b1 - d[1] * b0;
}

static void unit(float* d) {
  float inv = 1.0f / sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  d[0] = d[0] * inv;
  d[1] = d[1] * inv;
  d[2] = d[2] * inv;
}

static void electron(const world* w, stream* s, uint64_t* edep, float E, float* p, int* ix, float* d,
                     uint64_t* esc, uint64_t* nsteps) {
  float R = interp(w->range, w->nr, E / w->rde);
  for (int it = 0; it < 100000 && E > w->ecut; ++it) {
    *nsteps += 1;
    int64_t v = vox(w, ix[0], ix[1], ix[2]);
    float dens = rho_at(w, ix[0], ix[1], ix[2]);
    float vs[3] = {w->v0, w->v1, w->v2};
    float db = 3.0e38f;
    int ax = -1;
    for (int a = 0; a < 3; ++a) {
      if (d[a] > 0.0f) {
        float t = ((float)(ix[a] + 1) * vs[a] - p[a]) / d[a];
        if (t < db) { db = t; ax = a; }
      }
      if (d[a] < 0.0f) {
        float t = ((float)ix[a] * vs[a] - p[a]) / d[a];
        if (t < db) { db = t; ax = a; }
      }
    }
    if (db < 0.0f) db = 0.0f;
    float smax = 0.25f * R / dens;
    int cross = db <= smax;
    float st = cross ? db : smax;
    float t = dens * st;
    if (t >= R) {
      edep[v] += q32(E);
      E = 0.0f;
      break;
    }
    float Rn = R - t;
    float En = e_of_r(w, Rn);
    if (E > En) edep[v] += q32(E - En);
    for (int a = 0; a < 3; ++a) p[a] = p[a] + st * d[a];
    if (cross) {
      ix[ax] += (d[ax] > 0.0f) ? 1 : -1;
      if (ix[0] < 0 || ix[0] >= w->n0 || ix[1] < 0 || ix[1] >= w->n1 || ix[2] < 0 || ix[2] >= w->n2) {
        *esc += q32(En);
        E = 0.0f;
        break;
      }
    }
    float x = t / X0WATER;
    if (x > 1e-6f) {
      float Em = 0.5f * (E + En);
      float bcp = Em * (Em + 2.0f * MEC2) / (Em + MEC2);
      float fac = 1.0f + 0.038f * ln_f(x);
      if (fac < 0.0f) fac = 0.0f;
      float th0 = 13.6f / bcp * sqrtf(x) * fac;
      if (th0 > 0.0f) {
        float g1 = 0.0f, g2 = 0.0f;
        for (int k = 0; k < 64; ++k) {
          float a = 2.0f * unif(s) - 1.0f, b = 2.0f * unif(s) - 1.0f;
          float q = a * a + b * b;
          if (q < 1.0f && q > 0.0f) {
            float f = sqrtf(-2.0f * ln_f(q) / q);
            g1 = a * f;
            g2 = b * f;
            break;
          }
        }
        float e1[3], e2[3];
        perp(d, e1, e2);
        for (int a = 0; a < 3; ++a) d[a] = d[a] + th0 * (g1 * e1[a] + g2 * e2[a]);
        unit(d);
      }
    }
    E = En;
    R = Rn;
  }
  if (E > 0.0f) edep[vox(w, ix[0], ix[1], ix[2])] += q32(E);
}

static void photon(const world* w, stream* s, uint64_t* edep, float E, float* p, int* ix, float* d, uint64_t* esc,
                   uint64_t* nsteps) {
  float vs[3] = {w->v0, w->v1, w->v2};
  int nn[3] = {w->n0, w->n1, w->n2};
  for (int it = 0; it < 100000; ++it) {
    *nsteps += 1;
    if (E <= w->ecut) {
      edep[vox(w, ix[0], ix[1], ix[2])] += q32(E);
      return;
    }
    float mu = interp(w->mu, w->np, E / w->pde);
    float st = -ln_f(unif(s)) / (mu * w->rho_max);
    for (int a = 0; a < 3; ++a) p[a] = p[a] + st * d[a];
    float f[3];
    for (int a = 0; a < 3; ++a) f[a] = p[a] / vs[a];
    if (f[0] < 0.0f || f[1] < 0.0f || f[2] < 0.0f || f[0] >= (float)nn[0] || f[1] >= (float)nn[1] ||
        f[2] >= (float)nn[2]) {
      *esc += q32(E);
      return;
    }
    for (int a = 0; a < 3; ++a) {
      ix[a] = (int)f[a];
      if (ix[a] >= nn[a]) ix[a] = nn[a] - 1;
    }
    float dens = rho_at(w, ix[0], ix[1], ix[2]);
    if (unif(s) * w->rho_max > dens) continue;
    int64_t v = vox(w, ix[0], ix[1], ix[2]);
    float cf = interp(w->cf, w->np, E / w->pde);
    if (unif(s) > cf) {
      edep[v] += q32(E);
      return;
    }
    float k = E / MEC2;
    float eta = 1.0f;
    for (int r = 0; r < 1000; ++r) {
      float r1 = unif(s), r2 = unif(s), r3 = unif(s);
      if (r1 <= (1.0f + 2.0f * k) / (9.0f + 2.0f * k)) {
        float et = 1.0f + 2.0f * k * r2;
        if (r3 <= 4.0f * (1.0f / et - 1.0f / (et * et))) {
          eta = et;
          break;
        }
      } else {
        float et = (1.0f + 2.0f * k) / (1.0f + 2.0f * k * r2);
        float c = 1.0f - (et - 1.0f) / k;
        if (r3 <= 0.5f * (c * c + 1.0f / et)) {
          eta = et;
          break;
        }
      }
    }
    float En = E / eta;
    float c = 1.0f - (eta - 1.0f) / k;
    if (c > 1.0f) c = 1.0f;
    if (c < -1.0f) c = -1.0f;
    edep[v] += q32(E - En);
    float sn = sqrtf(1.0f - c * c);
    float ca = 1.0f, sa = 0.0f;
    for (int r = 0; r < 64; ++r) {
      float a = 2.0f * unif(s) - 1.0f, b = 2.0f * unif(s) - 1.0f;
      float q = a * a + b * b;
      if (q < 1.0f && q > 0.0f) {
        float inv = 1.0f / sqrtf(q);
        ca = a * inv;
        sa = b * inv;
        break;
      }
    }
    float e1[3], e2[3];
    perp(d, e1, e2);
    for (int a = 0; a < 3; ++a) d[a] = c * d[a] + sn * (ca * e1[a] + sa * e2[a]);
    unit(d);
    E = En;
  }
}

/* Runs histories [h_begin, h_end) and ADDS their deposits into edep (uint64, n voxels).
 * counters[0..3]: total source weight, emitted, escaped, steps (the last three added to).
 * Returns 0, or 1 if the activity sums to zero (nothing run). */
int pvd_mc_oracle_run(int n0, int n1, int n2, const double* voxel_mm, const float* act, const float* rho,
                      const float* beta, int nb, const float* range, int nr, float rde, const float* mu,
                      const float* cf, int np, float pde, int ng, const float* ge, const float* gp, float by,
                      float ecut, uint64_t seed, uint64_t h_begin, uint64_t h_end, uint64_t* edep,
                      uint64_t* counters) {
  int64_t n = (int64_t)n0 * n1 * n2;
  float amax = 0.0f, rmax = 0.0f;
  for (int64_t i = 0; i < n; ++i) {
    if (act[i] > amax) amax = act[i];
    if (rho && rho[i] > rmax) rmax = rho[i];
  }
  float scale = (amax > 0.0f) ? FIXS / amax : 0.0f;
  uint64_t* pre = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)n);
  uint64_t run = 0;
  for (int64_t i = 0; i < n; ++i) {
    float a = act[i];
    if (!(a > 0.0f)) a = 0.0f;
    run += (uint64_t)(a * scale);
    pre[i] = run;
  }
  counters[0] = run;
  if (run == 0) {
    free(pre);
    return 1;
  }
  world w = {beta, range, mu, cf, nb, nr, np, rde, pde, ng, ge, gp, by, ecut, n0, n1, n2,
             (float)(voxel_mm[0] * 0.1), (float)(voxel_mm[1] * 0.1), (float)(voxel_mm[2] * 0.1), rho,
             rho ? rmax : 1.0f};
  uint64_t emitted = 0, escaped = 0, steps = 0;
  for (uint64_t h = h_begin; h < h_end; ++h) {
    stream s;
    s.k0 = (uint32_t)seed;
    s.k1 = (uint32_t)(seed >> 32);
    s.h0 = (uint32_t)h;
    s.h1 = (uint32_t)(h >> 32);
    s.c = 0;
    s.u = 4;
    uint64_t hi = draw(&s);
    uint64_t r64 = (hi << 32) | draw(&s);
    uint64_t target = (uint64_t)(((unsigned __int128)r64 * run) >> 64);
    int64_t lo = 0, up = n - 1;
    while (lo < up) {
      int64_t mid = (lo + up) >> 1;
      if (pre[mid] > target)
        up = mid;
      else
        lo = mid + 1;
    }
    int c2 = (int)(lo % n2), c1 = (int)((lo / n2) % n1), c0 = (int)(lo / ((int64_t)n1 * n2));
    float p0 = ((float)c0 + unif(&s)) * w.v0;
    float p1 = ((float)c1 + unif(&s)) * w.v1;
    float p2 = ((float)c2 + unif(&s)) * w.v2;
    if (by > 0.0f && unif(&s) <= by) {
      float E = interp(beta, nb, unif(&s) * (float)(nb - 1));
      emitted += q32(E);
      float d[3], p[3] = {p0, p1, p2};
      int ix[3] = {c0, c1, c2};
      direction(&s, d);
      electron(&w, &s, edep, E, p, ix, d, &escaped, &steps);
    }
    for (int l = 0; l < ng; ++l) {
      if (unif(&s) <= gp[l]) {
        float E = ge[l];
        emitted += q32(E);
        float d[3], p[3] = {p0, p1, p2};
        int ix[3] = {c0, c1, c2};
        direction(&s, d);
        photon(&w, &s, edep, E, p, ix, d, &escaped, &steps);
      }
    }
  }
  counters[1] += emitted;
  counters[2] += escaped;
  counters[3] += steps;
  free(pre);
  return 0;
}

/* Philox4x32-10 of one counter block (exported for known-answer tests). */
void pvd_mc_oracle_philox(uint32_t* ctr4, const uint32_t* key2) { philox10(ctr4, key2[0], key2[1]); }
