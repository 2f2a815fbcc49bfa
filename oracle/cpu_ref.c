/*
 * cpu_ref.c — C/OpenMP restatement of BAOrec.jl's CPU hot loops (test
 * infrastructure: the timed CPU baseline, never the product).
 *
 * Follows the reference's CPU methods (paths inside the BAOrec.jl project):
 *   cic_paint   src/mas.jl:1-52        serial loop, as the reference's cic!
 *   read_cic    src/mas.jl:218-269     threaded gather
 *   jacobi      src/multigrid.jl:14-135 damped Jacobi (ω, ν sweeps)
 *   residual    src/multigrid.jl:213-326
 *   reduce      src/multigrid.jl:520-584 full-weighting restriction
 *   prolong     src/multigrid.jl:398-453 trilinear prolongation
 * Meshes are x-fastest FP32 arrays: (ix, iy, iz) at ix + n1*(iy + n2*iz).
 * FFTs and element-wise k-space work are done by the Python driver
 * (oracle/cpu_port.py) with scipy.fft.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define IDX(i, j, k) ((size_t)(i) + (size_t)n1 * ((size_t)(j) + (size_t)n2 * (size_t)(k)))

int cpu_threads(void) {
#ifdef _OPENMP
  extern int omp_get_max_threads(void);
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* cic! CPU method; returns -1 on the reference's BoundsError. */
int cic_paint(float* rho, int n1, int n2, int n3, float* x, float* y, float* z, const float* w, int64_t np,
              const float* L, const float* bmin, int wrap) {
  const int n[3] = {n1, n2, n3};
  for (int64_t i = 0; i < np; ++i) {
    if (wrap) {
      x[i] = (x[i] - bmin[0]) > L[0] ? x[i] - L[0] : x[i];
      y[i] = (y[i] - bmin[0]) > L[0] ? y[i] - L[0] : y[i];
      z[i] = (z[i] - bmin[0]) > L[0] ? z[i] - L[0] : z[i];
    }
    float p[3] = {x[i], y[i], z[i]};
    int c0[3], c1[3];
    float w0[3], w1[3];
    for (int a = 0; a < 3; ++a) {
      float g = (p[a] - bmin[a]) * (float)n[a] / L[a] + 1.0f;   /* built with -ffp-contract=off */
      int c = (int)floorf(g);
      w1[a] = g - (float)c;
      w0[a] = 1.0f - w1[a];
      if (c == n[a] + 1) c = 1;
      int u = (c == n[a] && wrap) ? 1 : c + 1;
      if (c < 1 || c > n[a] || u < 1 || u > n[a]) return -1;
      c0[a] = c - 1;
      c1[a] = u - 1;
    }
    w0[0] *= w[i];
    w1[0] *= w[i];
    rho[IDX(c0[0], c0[1], c0[2])] += w0[0] * w0[1] * w0[2];
    rho[IDX(c1[0], c0[1], c0[2])] += w1[0] * w0[1] * w0[2];
    rho[IDX(c0[0], c1[1], c0[2])] += w0[0] * w1[1] * w0[2];
    rho[IDX(c0[0], c0[1], c1[2])] += w0[0] * w0[1] * w1[2];
    rho[IDX(c1[0], c1[1], c0[2])] += w1[0] * w1[1] * w0[2];
    rho[IDX(c1[0], c0[1], c1[2])] += w1[0] * w0[1] * w1[2];
    rho[IDX(c0[0], c1[1], c1[2])] += w0[0] * w1[1] * w1[2];
    rho[IDX(c1[0], c1[1], c1[2])] += w1[0] * w1[1] * w1[2];
  }
  return 0;
}

/* read_cic! CPU method (wrap = true). */
int read_cic(const float* f, int n1, int n2, int n3, const float* x, const float* y, const float* z, int64_t np,
             const float* L, const float* bmin, float* out) {
  const int n[3] = {n1, n2, n3};
  float cell[3];
  for (int a = 0; a < 3; ++a) cell[a] = L[a] / (float)n[a];
  int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
  for (int64_t i = 0; i < np; ++i) {
    const float p[3] = {x[i], y[i], z[i]};
    int lo[3], hi[3];
    float d[3], u[3];
    for (int a = 0; a < 3; ++a) {
      float dist = (p[a] - bmin[a]) / cell[a];
      int c = (int)floorf(dist);
      u[a] = dist - (float)c;
      d[a] = 1.0f - u[a];
      c += 1;
      int l = c > n[a] ? c - n[a] : c;
      int h = l + 1;
      h = h > n[a] ? h - n[a] : h;
      if (l < 1 || h > n[a]) bad = 1;
      lo[a] = l - 1;
      hi[a] = h - 1;
    }
    if (bad) { out[i] = NAN; continue; }
    out[i] = f[IDX(lo[0], lo[1], lo[2])] * d[0] * d[1] * d[2] + f[IDX(lo[0], lo[1], hi[2])] * d[0] * d[1] * u[2] +
             f[IDX(lo[0], hi[1], lo[2])] * d[0] * u[1] * d[2] + f[IDX(lo[0], hi[1], hi[2])] * d[0] * u[1] * u[2] +
             f[IDX(hi[0], lo[1], lo[2])] * u[0] * d[1] * d[2] + f[IDX(hi[0], lo[1], hi[2])] * u[0] * d[1] * u[2] +
             f[IDX(hi[0], hi[1], lo[2])] * u[0] * u[1] * d[2] + f[IDX(hi[0], hi[1], hi[2])] * u[0] * u[1] * u[2];
  }
  return bad ? -1 : 0;
}

typedef struct {
  float cell2[3], icell2[3], pg[3], beta;
  const float* P[3];
  int local;
} geom_t;

static inline void coef(const geom_t* G, int i, int j, int k, float* gp, float* g, float* p) {
  if (G->local) { p[0] = G->P[0][i]; p[1] = G->P[1][j]; p[2] = G->P[2][k]; }
  else { p[0] = G->pg[0]; p[1] = G->pg[1]; p[2] = G->pg[2]; }
  *g = G->beta / (G->cell2[0] * (p[0] * p[0]) + G->cell2[1] * (p[1] * p[1]) + G->cell2[2] * (p[2] * p[2]));
  for (int a = 0; a < 3; ++a) gp[a] = G->icell2[a] + *g * (p[a] * p[a]);
}

static void geom_init(geom_t* G, int n1, int n2, int n3, const float* L, const float* P0, const float* P1,
                      const float* P2, const float* los, float beta) {
  const int n[3] = {n1, n2, n3};
  for (int a = 0; a < 3; ++a) {
    float cell = L[a] / (float)n[a];
    G->cell2[a] = cell * cell;
    G->icell2[a] = 1.0f / G->cell2[a];
    G->pg[a] = los ? los[a] / cell : 0.0f;
  }
  G->P[0] = P0; G->P[1] = P1; G->P[2] = P2;
  G->local = los == NULL;
  G->beta = beta;
}

/* neighbour bracket of src/multigrid.jl:64-79 */
static inline float bracket(const float* v, int n1, int n2, int n3, int i, int j, int k, const float* gp, float g,
                            const float* p, int local) {
  int ip = i + 1 == n1 ? 0 : i + 1, im = i == 0 ? n1 - 1 : i - 1;
  int jp = j + 1 == n2 ? 0 : j + 1, jm = j == 0 ? n2 - 1 : j - 1;
  int kp = k + 1 == n3 ? 0 : k + 1, km = k == 0 ? n3 - 1 : k - 1;
  float s = gp[0] * (v[IDX(ip, j, k)] + v[IDX(im, j, k)]) + gp[1] * (v[IDX(i, jp, k)] + v[IDX(i, jm, k)]) +
            gp[2] * (v[IDX(i, j, kp)] + v[IDX(i, j, km)]) +
            g / 2 * (p[0] * p[1] * (v[IDX(ip, jp, k)] + v[IDX(im, jm, k)] - v[IDX(im, jp, k)] - v[IDX(ip, jm, k)]) +
                     p[0] * p[2] * (v[IDX(ip, j, kp)] + v[IDX(im, j, km)] - v[IDX(im, j, kp)] - v[IDX(ip, j, km)]) +
                     p[1] * p[2] * (v[IDX(i, jp, kp)] + v[IDX(i, jm, km)] - v[IDX(i, jm, kp)] - v[IDX(i, jp, km)]));
  if (local)
    s += g * (p[0] * (v[IDX(ip, j, k)] - v[IDX(im, j, k)]) + p[1] * (v[IDX(i, jp, k)] - v[IDX(i, jm, k)]) +
              p[2] * (v[IDX(i, j, kp)] - v[IDX(i, j, km)]));
  return s;
}

/* jacobi!: niter damped sweeps; tmp is a scratch mesh. */
void jacobi(float* v, const float* f, float* tmp, int n1, int n2, int n3, const float* L, const float* P0,
            const float* P1, const float* P2, const float* los, float beta, float omega, int niter) {
  geom_t G;
  geom_init(&G, n1, n2, n3, L, P0, P1, P2, los, beta);
  for (int it = 0; it < niter; ++it) {
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 0; k < n3; ++k)
      for (int j = 0; j < n2; ++j)
        for (int i = 0; i < n1; ++i) {
          float gp[3], g, p[3];
          coef(&G, i, j, k, gp, &g, p);
          float jac = f[IDX(i, j, k)] + bracket(v, n1, n2, n3, i, j, k, gp, g, p, G.local);
          tmp[IDX(i, j, k)] = jac / (2 * (gp[0] + gp[1] + gp[2]));
        }
    size_t N = (size_t)n1 * n2 * n3;
#pragma omp parallel for schedule(static)
    for (size_t e = 0; e < N; ++e) v[e] = (1 - omega) * v[e] + omega * tmp[e];
  }
}

void residual(float* r, const float* v, const float* f, int n1, int n2, int n3, const float* L, const float* P0,
              const float* P1, const float* P2, const float* los, float beta) {
  geom_t G;
  geom_init(&G, n1, n2, n3, L, P0, P1, P2, los, beta);
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < n3; ++k)
    for (int j = 0; j < n2; ++j)
      for (int i = 0; i < n1; ++i) {
        float gp[3], g, p[3];
        coef(&G, i, j, k, gp, &g, p);
        float av = 2 * (gp[0] + gp[1] + gp[2]) * v[IDX(i, j, k)] - bracket(v, n1, n2, n3, i, j, k, gp, g, p, G.local);
        r[IDX(i, j, k)] = f[IDX(i, j, k)] - av;
      }
}

/* reduce!: fine (n1,n2,n3) → coarse (n1/2, n2/2, n3/2) */
void reduce(float* c, const float* v, int n1, int n2, int n3) {
  const int c1 = n1 / 2, c2 = n2 / 2, c3 = n3 / 2;
#pragma omp parallel for collapse(2) schedule(static)
  for (int ck = 0; ck < c3; ++ck)
    for (int cj = 0; cj < c2; ++cj)
      for (int ci = 0; ci < c1; ++ci) {
        int i = 2 * ci + 1, j = 2 * cj + 1, k = 2 * ck + 1;
        int ip = i + 1 == n1 ? 0 : i + 1, im = i - 1, jp = j + 1 == n2 ? 0 : j + 1, jm = j - 1;
        int kp = k + 1 == n3 ? 0 : k + 1, km = k - 1;
#define F(a, b, d) v[IDX(a, b, d)]
        float s = 8 * F(i, j, k) + 4 * (F(ip, j, k) + F(im, j, k) + F(i, jp, k) + F(i, jm, k) + F(i, j, kp) + F(i, j, km)) +
                  2 * (F(ip, jp, k) + F(im, jp, k) + F(ip, jm, k) + F(im, jm, k) + F(ip, j, kp) + F(im, j, kp) +
                       F(ip, j, km) + F(im, j, km) + F(i, jp, kp) + F(i, jm, kp) + F(i, jp, km) + F(i, jm, km)) +
                  F(ip, jp, kp) + F(im, jp, kp) + F(ip, jm, kp) + F(im, jm, kp) + F(ip, jp, km) + F(im, jp, km) +
                  F(ip, jm, km) + F(im, jm, km);
#undef F
        c[(size_t)ci + (size_t)c1 * ((size_t)cj + (size_t)c2 * ck)] = s / 64.0f;
      }
}

/* prolong!: coarse → fine (n1,n2,n3 = fine size); add != 0 adds into v. */
void prolong(float* v, const float* c, int n1, int n2, int n3, int add) {
  const int c1 = n1 / 2, c2 = n2 / 2, c3 = n3 / 2;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < c3; ++k)
    for (int j = 0; j < c2; ++j)
      for (int i = 0; i < c1; ++i) {
        int ip = i + 1 == c1 ? 0 : i + 1, jp = j + 1 == c2 ? 0 : j + 1, kp = k + 1 == c3 ? 0 : k + 1;
#define C(a, b, d) c[(size_t)(a) + (size_t)c1 * ((size_t)(b) + (size_t)c2 * (d))]
        float c000 = C(i, j, k), c100 = C(ip, j, k), c010 = C(i, jp, k), c001 = C(i, j, kp);
        float c110 = C(ip, jp, k), c011 = C(i, jp, kp), c101 = C(ip, j, kp), c111 = C(ip, jp, kp);
#undef C
        int x0 = 2 * i + 1, y0 = 2 * j + 1, z0 = 2 * k + 1;
        int x1 = x0 + 1 == n1 ? 0 : x0 + 1, y1 = y0 + 1 == n2 ? 0 : y0 + 1, z1 = z0 + 1 == n3 ? 0 : z0 + 1;
        float val[8] = {c000, (c000 + c100) / 2, (c000 + c010) / 2, (c000 + c001) / 2,
                        (c000 + c100 + c010 + c110) / 4, (c000 + c010 + c001 + c011) / 4,
                        (c000 + c100 + c001 + c101) / 4,
                        (c000 + c100 + c010 + c001 + c110 + c101 + c011 + c111) / 8};
        size_t o[8] = {IDX(x0, y0, z0), IDX(x1, y0, z0), IDX(x0, y1, z0), IDX(x0, y0, z1),
                       IDX(x1, y1, z0), IDX(x0, y1, z1), IDX(x1, y0, z1), IDX(x1, y1, z1)};
        for (int q = 0; q < 8; ++q) v[o[q]] = add ? v[o[q]] + val[q] : val[q];
      }
}

/* A v in FP64 arithmetic with the FP32 coefficients of src/multigrid.jl:17-29,
 * 55-62 (computed in FP32 by coef(), exactly as the FP32 restatement rounds
 * them) and the operator of src/multigrid.jl:262-276: 2 Σ gp_i v - bracket.
 * This is the accuracy judge's operator: the FP64 solution of the same
 * discrete system the FP32 code solves. */
void apply_op_f64(double* out, const double* v, int n1, int n2, int n3, const float* L, const float* P0,
                  const float* P1, const float* P2, const float* los, float beta) {
  geom_t G;
  geom_init(&G, n1, n2, n3, L, P0, P1, P2, los, beta);
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < n3; ++k)
    for (int j = 0; j < n2; ++j)
      for (int i = 0; i < n1; ++i) {
        float gpf[3], gf, pf[3];
        coef(&G, i, j, k, gpf, &gf, pf);
        const double gp0 = gpf[0], gp1 = gpf[1], gp2 = gpf[2], g = gf, p0 = pf[0], p1 = pf[1], p2 = pf[2];
        int ip = i + 1 == n1 ? 0 : i + 1, im = i == 0 ? n1 - 1 : i - 1;
        int jp = j + 1 == n2 ? 0 : j + 1, jm = j == 0 ? n2 - 1 : j - 1;
        int kp = k + 1 == n3 ? 0 : k + 1, km = k == 0 ? n3 - 1 : k - 1;
        double s = gp0 * (v[IDX(ip, j, k)] + v[IDX(im, j, k)]) + gp1 * (v[IDX(i, jp, k)] + v[IDX(i, jm, k)]) +
                   gp2 * (v[IDX(i, j, kp)] + v[IDX(i, j, km)]) +
                   g / 2 * (p0 * p1 * (v[IDX(ip, jp, k)] + v[IDX(im, jm, k)] - v[IDX(im, jp, k)] - v[IDX(ip, jm, k)]) +
                            p0 * p2 * (v[IDX(ip, j, kp)] + v[IDX(im, j, km)] - v[IDX(im, j, kp)] - v[IDX(ip, j, km)]) +
                            p1 * p2 * (v[IDX(i, jp, kp)] + v[IDX(i, jm, km)] - v[IDX(i, jm, kp)] - v[IDX(i, jp, km)]));
        if (G.local)
          s += g * (p0 * (v[IDX(ip, j, k)] - v[IDX(im, j, k)]) + p1 * (v[IDX(i, jp, k)] - v[IDX(i, jm, k)]) +
                    p2 * (v[IDX(i, j, kp)] - v[IDX(i, j, km)]));
        out[IDX(i, j, k)] = 2 * (gp0 + gp1 + gp2) * v[IDX(i, j, k)] - s;
      }
}
