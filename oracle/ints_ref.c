/*
 * ints_ref.c -- plain-C restatement of the molecular integrals of the oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  Like the rest of oracle/ this is the checker: it
 * is built by build() into oracle/_build/libints_ref.so and called through
 * ctypes by oracle/molecule.py (ao_integrals_c) and the fixture scripts.  The
 * product never links or loads it.
 *
 * It computes the same integrals as oracle/molecule.py (one_electron,
 * two_electron, _transform), scalar and unoptimised, so that systems with a
 * few hundred basis functions -- (H2O)10 in cc-pVDZ has 240 -- can be handled
 * on the CPU: overlap, kinetic energy, nuclear attraction and electron
 * repulsion integrals over contracted Cartesian Gaussians by the
 * McMurchie-Davidson scheme (L. E. McMurchie, E. R. Davidson, J. Comput.
 * Phys. 26, 218 (1978)):
 *   Hermite expansion coefficients E_t^{ij} by the two-term recurrences of
 *   the product of two 1-D Gaussians;
 *   Hermite Coulomb integrals R_{tuv} from the Boys function
 *   F_n(T) = int_0^1 u^{2n} exp(-T u^2) du by the R^{n}_{t+1,u,v} =
 *   t R^{n+1}_{t-1,u,v} + X_PQ R^{n+1}_{t,u,v} recurrences;
 *   (ab|cd) = 2 pi^{5/2} / (p q sqrt(p+q)) sum E^{ab}_{tuv} (-1)^{tau+nu+phi}
 *   E^{cd}_{tau nu phi} R_{t+tau,u+nu,v+phi}(alpha, P - Q).
 * The Boys function is evaluated from its convergent series
 * F_n(T) = e^{-T} sum_k (2T)^k / ((2n+1)(2n+3)...(2n+2k+1)) for T <= 50 and
 * from F_0 = (pi/T)^{1/2} / 2 with the upward recurrence above it (where
 * e^{-T} < 2e-22).
 *
 * In the reference these integrals come from Libint2 (not part of the MPQC
 * tree; src/mpqc/chemistry/qc/lcao/integrals/make_engine.h:24-88 creates the
 * engines); the basis sets are those of oracle/molecule.py.  Results are in
 * the spherical basis of oracle/molecule.py (d shells: xy, yz, 2zz-xx-yy, xz,
 * xx-yy, unnormalised; the caller rescales to unit self-overlap) and follow
 * its Cartesian order (x-major) for p shells.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define LMAX 2
#define LE (2 * LMAX + 2)   /* 1-D E indices up to lb + 2 (kinetic) */
#define LR (4 * LMAX)        /* highest Hermite order of an ERI       */

static const double PI = 3.14159265358979323846;

static void boys(int nmax, double T, double *F) {
  if (T > 50.0) {
    F[0] = 0.5 * sqrt(PI / T);
    const double e = exp(-T);
    for (int n = 0; n < nmax; ++n) F[n + 1] = ((2 * n + 1) * F[n] - e) / (2.0 * T);
    return;
  }
  const double e = exp(-T);
  double term = 1.0 / (2 * nmax + 1), sum = term;
  for (int k = 1; k < 400; ++k) {
    term *= 2.0 * T / (2 * nmax + 2 * k + 1);
    sum += term;
    if (term < 1e-18 * sum) break;
  }
  F[nmax] = e * sum;
  for (int n = nmax - 1; n >= 0; --n) F[n] = (2.0 * T * F[n + 1] + e) / (2 * n + 1);
}

/* E[i][j][t], i <= la, j <= lb, t <= i + j (1-D, one primitive pair) */
static void hermite_e(int la, int lb, double a, double b, double xab, double E[LE + 1][LE + 1][2 * LE + 2]) {
  const double p = a + b, mu = a * b / p;
  const double xpa = -b / p * xab, xpb = a / p * xab, hp = 0.5 / p;
  memset(E, 0, sizeof(double) * (LE + 1) * (LE + 1) * (2 * LE + 2));
  E[0][0][0] = exp(-mu * xab * xab);
  for (int i = 0; i <= la; ++i)
    for (int j = 0; j <= lb; ++j) {
      if (i == 0 && j == 0) continue;
      int ii, jj;
      double x;
      const double *src;
      if (i > 0) {
        ii = i - 1, jj = j, x = xpa, src = E[i - 1][j];
      } else {
        ii = i, jj = j - 1, x = xpb, src = E[i][j - 1];
      }
      for (int t = 0; t <= ii + jj + 1; ++t) {
        double v = x * src[t];
        if (t > 0) v += hp * src[t - 1];
        if (t + 1 <= ii + jj) v += (t + 1) * src[t + 1];
        E[i][j][t] = v;
      }
    }
}

/* R[t][u][v] = R^0_{tuv}(alpha, (X, Y, Z)) for t + u + v <= L */
static void hermite_r(int L, double alpha, double X, double Y, double Z, double R[LR + 1][LR + 1][LR + 1]) {
  static __thread double Rn[LR + 1][LR + 1][LR + 1][LR + 1];
  double F[LR + 1];
  boys(L, alpha * (X * X + Y * Y + Z * Z), F);
  double m = 1.0;
  for (int n = 0; n <= L; ++n) {
    Rn[n][0][0][0] = m * F[n];
    m *= -2.0 * alpha;
  }
  for (int tot = 1; tot <= L; ++tot)
    for (int n = 0; n <= L - tot; ++n)
      for (int t = 0; t <= tot; ++t)
        for (int u = 0; u <= tot - t; ++u) {
          const int v = tot - t - u;
          double val;
          if (t > 0) {
            val = X * Rn[n + 1][t - 1][u][v];
            if (t > 1) val += (t - 1) * Rn[n + 1][t - 2][u][v];
          } else if (u > 0) {
            val = Y * Rn[n + 1][t][u - 1][v];
            if (u > 1) val += (u - 1) * Rn[n + 1][t][u - 2][v];
          } else {
            val = Z * Rn[n + 1][t][u][v - 1];
            if (v > 1) val += (v - 1) * Rn[n + 1][t][u][v - 2];
          }
          Rn[n][t][u][v] = val;
        }
  for (int t = 0; t <= L; ++t)
    for (int u = 0; u <= L - t; ++u)
      for (int v = 0; v <= L - t - u; ++v) R[t][u][v] = Rn[0][t][u][v];
}

static int ncart(int l) { return (l + 1) * (l + 2) / 2; }
static int nfunc(int l, int pure) { return (pure && l >= 2) ? 2 * l + 1 : ncart(l); }

/* Cartesian components (i, j, k), i + j + k = l, x-major */
static void comps(int l, int c[][3]) {
  int n = 0;
  for (int i = l; i >= 0; --i)
    for (int j = l - i; j >= 0; --j) {
      c[n][0] = i;
      c[n][1] = j;
      c[n][2] = l - i - j;
      ++n;
    }
}

/* rows of the spherical d functions over the Cartesian components
   xx, xy, xz, yy, yz, zz */
static const double PURE_D[5][6] = {
    {0, 1, 0, 0, 0, 0}, {0, 0, 0, 0, 1, 0}, {-1, 0, 0, -1, 0, 2}, {0, 0, 1, 0, 0, 0}, {1, 0, 0, -1, 0, 0}};

/* out[nf] <- T x[nc] for one index of a shell */
static double tmat(int l, int pure, int f, int c) {
  if (pure && l == 2) return PURE_D[f][c];
  return f == c ? 1.0 : 0.0;
}

typedef struct {
  int l, nprim, pure, off;       /* off: first spherical function */
  const double *exps, *coefs;    /* coefs include the primitive normalisation */
  double c[3];
} shell_t;

static shell_t *make_shells(int nshell, const int *l, const double *center, const int *nprim, const double *exps,
                            const double *coefs, int pure, int *nf_out) {
  shell_t *s = (shell_t *)malloc(sizeof(shell_t) * (size_t)nshell);
  int off = 0, po = 0;
  for (int k = 0; k < nshell; ++k) {
    s[k].l = l[k];
    s[k].nprim = nprim[k];
    s[k].pure = pure;
    s[k].off = off;
    s[k].exps = exps + po;
    s[k].coefs = coefs + po;
    for (int x = 0; x < 3; ++x) s[k].c[x] = center[3 * k + x];
    off += nfunc(l[k], pure);
    po += nprim[k];
  }
  *nf_out = off;
  return s;
}

/* S, T (kinetic) and V (nuclear attraction) in the spherical basis, each nf x nf */
int oneint_sph(int nshell, const int *l, const double *center, const int *nprim, const double *exps,
               const double *coefs, int pure, int natom, const double *Zn, const double *xyz, double *S, double *Tk,
               double *V) {
  int nf;
  shell_t *sh = make_shells(nshell, l, center, nprim, exps, coefs, pure, &nf);
#pragma omp parallel for schedule(dynamic)
  for (int A = 0; A < nshell; ++A) {
    double E[3][LE + 1][LE + 1][2 * LE + 2];
    double R[LR + 1][LR + 1][LR + 1];
    int ca[6][3], cb[6][3];
    for (int B = 0; B < nshell; ++B) {
      const shell_t *a = &sh[A], *b = &sh[B];
      const int na = ncart(a->l), nb = ncart(b->l);
      comps(a->l, ca);
      comps(b->l, cb);
      double s[6][6], t[6][6], v[6][6];
      memset(s, 0, sizeof s);
      memset(t, 0, sizeof t);
      memset(v, 0, sizeof v);
      for (int i = 0; i < a->nprim; ++i)
        for (int j = 0; j < b->nprim; ++j) {
          const double ea = a->exps[i], eb = b->exps[j], p = ea + eb;
          const double cw = a->coefs[i] * b->coefs[j];
          for (int x = 0; x < 3; ++x) hermite_e(a->l, b->l + 2, ea, eb, a->c[x] - b->c[x], E[x]);
          const double sq = sqrt(PI / p);
          double P[3];
          for (int x = 0; x < 3; ++x) P[x] = (ea * a->c[x] + eb * b->c[x]) / p;
          for (int ia = 0; ia < na; ++ia)
            for (int ib = 0; ib < nb; ++ib) {
              double s1[3], t1[3];
              for (int x = 0; x < 3; ++x) {
                const int i1 = ca[ia][x], j1 = cb[ib][x];
                s1[x] = E[x][i1][j1][0] * sq;
                double tv = -2.0 * eb * eb * E[x][i1][j1 + 2][0] * sq + eb * (2 * j1 + 1) * s1[x];
                if (j1 >= 2) tv -= 0.5 * j1 * (j1 - 1) * E[x][i1][j1 - 2][0] * sq;
                t1[x] = tv;
              }
              s[ia][ib] += cw * s1[0] * s1[1] * s1[2];
              t[ia][ib] += cw * (t1[0] * s1[1] * s1[2] + s1[0] * t1[1] * s1[2] + s1[0] * s1[1] * t1[2]);
            }
          const int L = a->l + b->l;
          for (int C = 0; C < natom; ++C) {
            hermite_r(L, p, P[0] - xyz[3 * C], P[1] - xyz[3 * C + 1], P[2] - xyz[3 * C + 2], R);
            for (int ia = 0; ia < na; ++ia)
              for (int ib = 0; ib < nb; ++ib) {
                double h = 0.0;
                const int *u = ca[ia], *w = cb[ib];
                for (int tt = 0; tt <= u[0] + w[0]; ++tt)
                  for (int uu = 0; uu <= u[1] + w[1]; ++uu)
                    for (int vv = 0; vv <= u[2] + w[2]; ++vv)
                      h += E[0][u[0]][w[0]][tt] * E[1][u[1]][w[1]][uu] * E[2][u[2]][w[2]][vv] * R[tt][uu][vv];
                v[ia][ib] -= Zn[C] * cw * 2.0 * PI / p * h;
              }
          }
        }
      const int fa = nfunc(a->l, a->pure), fb = nfunc(b->l, b->pure);
      for (int f = 0; f < fa; ++f)
        for (int g = 0; g < fb; ++g) {
          double ss = 0, tt = 0, vv = 0;
          for (int ia = 0; ia < na; ++ia)
            for (int ib = 0; ib < nb; ++ib) {
              const double m = tmat(a->l, a->pure, f, ia) * tmat(b->l, b->pure, g, ib);
              if (m == 0.0) continue;
              ss += m * s[ia][ib];
              tt += m * t[ia][ib];
              vv += m * v[ia][ib];
            }
          const size_t k = (size_t)(a->off + f) * nf + (b->off + g);
          S[k] = ss;
          Tk[k] = tt;
          V[k] = vv;
        }
    }
  }
  free(sh);
  return nf;
}

/* (mu nu|la si) in the spherical basis, G[nf][nf][nf][nf], every element
   written (8-fold permutational symmetry). */
int eri_sph(int nshell, const int *l, const double *center, const int *nprim, const double *exps,
            const double *coefs, int pure, double *G) {
  int nf;
  shell_t *sh = make_shells(nshell, l, center, nprim, exps, coefs, pure, &nf);
  const long npair = (long)nshell * (nshell + 1) / 2;
  int *pa = (int *)malloc(sizeof(int) * (size_t)npair), *pb = (int *)malloc(sizeof(int) * (size_t)npair);
  long q = 0;
  for (int a = 0; a < nshell; ++a)
    for (int b = 0; b <= a; ++b) {
      pa[q] = a;
      pb[q] = b;
      ++q;
    }
  const size_t n1 = (size_t)nf, n2 = n1 * n1, n3 = n2 * n1;
#pragma omp parallel for schedule(dynamic, 1)
  for (long ip = npair - 1; ip >= 0; --ip) {
    double Eab[3][LE + 1][LE + 1][2 * LE + 2], Ecd[3][LE + 1][LE + 1][2 * LE + 2];
    double R[LR + 1][LR + 1][LR + 1];
    static __thread double blk[6][6][6][6], W[LR + 1][LR + 1][LR + 1];
    static __thread double sph[6][6][6][6], tmp[6][6][6][6];
    int ca[6][3], cb[6][3], cc[6][3], cd[6][3];
    const shell_t *A = &sh[pa[ip]], *B = &sh[pb[ip]];
    comps(A->l, ca);
    comps(B->l, cb);
    const int na = ncart(A->l), nb = ncart(B->l);
    const int Lab = A->l + B->l;
    for (long jp = 0; jp <= ip; ++jp) {
      const shell_t *C = &sh[pa[jp]], *D = &sh[pb[jp]];
      comps(C->l, cc);
      comps(D->l, cd);
      const int nc = ncart(C->l), nd = ncart(D->l);
      const int Lcd = C->l + D->l, L = Lab + Lcd;
      memset(blk, 0, sizeof blk);
      for (int i = 0; i < A->nprim; ++i)
        for (int j = 0; j < B->nprim; ++j) {
          const double a = A->exps[i], b = B->exps[j], p = a + b;
          const double cab = A->coefs[i] * B->coefs[j];
          double P[3];
          for (int x = 0; x < 3; ++x) {
            hermite_e(A->l, B->l, a, b, A->c[x] - B->c[x], Eab[x]);
            P[x] = (a * A->c[x] + b * B->c[x]) / p;
          }
          for (int k = 0; k < C->nprim; ++k)
            for (int m = 0; m < D->nprim; ++m) {
              const double c = C->exps[k], d = D->exps[m], qq = c + d;
              const double ccd = C->coefs[k] * D->coefs[m];
              double Q[3];
              for (int x = 0; x < 3; ++x) {
                hermite_e(C->l, D->l, c, d, C->c[x] - D->c[x], Ecd[x]);
                Q[x] = (c * C->c[x] + d * D->c[x]) / qq;
              }
              const double alpha = p * qq / (p + qq);
              hermite_r(L, alpha, P[0] - Q[0], P[1] - Q[1], P[2] - Q[2], R);
              const double pref = 2.0 * pow(PI, 2.5) / (p * qq * sqrt(p + qq)) * cab * ccd;
              for (int ic = 0; ic < nc; ++ic)
                for (int id = 0; id < nd; ++id) {
                  const int *u = cc[ic], *w = cd[id];
                  /* W[t][u][v] = sum (-1)^{tau+nu+phi} E^{cd} R[t+tau][u+nu][v+phi], t+u+v <= Lab */
                  for (int t = 0; t <= Lab; ++t)
                    for (int uu = 0; uu <= Lab - t; ++uu)
                      for (int vv = 0; vv <= Lab - t - uu; ++vv) {
                        double acc = 0.0;
                        for (int x = 0; x <= u[0] + w[0]; ++x)
                          for (int y = 0; y <= u[1] + w[1]; ++y)
                            for (int z = 0; z <= u[2] + w[2]; ++z) {
                              const double e = Ecd[0][u[0]][w[0]][x] * Ecd[1][u[1]][w[1]][y] * Ecd[2][u[2]][w[2]][z];
                              acc += (((x + y + z) & 1) ? -e : e) * R[t + x][uu + y][vv + z];
                            }
                        W[t][uu][vv] = acc;
                      }
                  for (int ia = 0; ia < na; ++ia)
                    for (int ib = 0; ib < nb; ++ib) {
                      const int *s1 = ca[ia], *s2 = cb[ib];
                      double acc = 0.0;
                      for (int t = 0; t <= s1[0] + s2[0]; ++t)
                        for (int uu = 0; uu <= s1[1] + s2[1]; ++uu)
                          for (int vv = 0; vv <= s1[2] + s2[2]; ++vv)
                            acc += Eab[0][s1[0]][s2[0]][t] * Eab[1][s1[1]][s2[1]][uu] * Eab[2][s1[2]][s2[2]][vv] *
                                   W[t][uu][vv];
                      blk[ia][ib][ic][id] += pref * acc;
                    }
                }
            }
        }
      /* spherical transform, one index at a time */
      const int fa = nfunc(A->l, A->pure), fb = nfunc(B->l, B->pure), fc = nfunc(C->l, C->pure),
                fd = nfunc(D->l, D->pure);
      memset(tmp, 0, sizeof tmp);
      for (int f = 0; f < fa; ++f)
        for (int x = 0; x < na; ++x) {
          const double m = tmat(A->l, A->pure, f, x);
          if (m == 0.0) continue;
          for (int ib = 0; ib < nb; ++ib)
            for (int ic = 0; ic < nc; ++ic)
              for (int id = 0; id < nd; ++id) tmp[f][ib][ic][id] += m * blk[x][ib][ic][id];
        }
      memset(blk, 0, sizeof blk);
      for (int f = 0; f < fa; ++f)
        for (int g = 0; g < fb; ++g)
          for (int x = 0; x < nb; ++x) {
            const double m = tmat(B->l, B->pure, g, x);
            if (m == 0.0) continue;
            for (int ic = 0; ic < nc; ++ic)
              for (int id = 0; id < nd; ++id) blk[f][g][ic][id] += m * tmp[f][x][ic][id];
          }
      memset(tmp, 0, sizeof tmp);
      for (int f = 0; f < fa; ++f)
        for (int g = 0; g < fb; ++g)
          for (int h = 0; h < fc; ++h)
            for (int x = 0; x < nc; ++x) {
              const double m = tmat(C->l, C->pure, h, x);
              if (m == 0.0) continue;
              for (int id = 0; id < nd; ++id) tmp[f][g][h][id] += m * blk[f][g][x][id];
            }
      memset(sph, 0, sizeof sph);
      for (int f = 0; f < fa; ++f)
        for (int g = 0; g < fb; ++g)
          for (int h = 0; h < fc; ++h)
            for (int e = 0; e < fd; ++e)
              for (int x = 0; x < nd; ++x) {
                const double m = tmat(D->l, D->pure, e, x);
                if (m != 0.0) sph[f][g][h][e] += m * tmp[f][g][h][x];
              }
      for (int f = 0; f < fa; ++f)
        for (int g = 0; g < fb; ++g)
          for (int h = 0; h < fc; ++h)
            for (int e = 0; e < fd; ++e) {
              const size_t i0 = A->off + f, j0 = B->off + g, k0 = C->off + h, l0 = D->off + e;
              const double val = sph[f][g][h][e];
              G[i0 * n3 + j0 * n2 + k0 * n1 + l0] = val;
              G[j0 * n3 + i0 * n2 + k0 * n1 + l0] = val;
              G[i0 * n3 + j0 * n2 + l0 * n1 + k0] = val;
              G[j0 * n3 + i0 * n2 + l0 * n1 + k0] = val;
              G[k0 * n3 + l0 * n2 + i0 * n1 + j0] = val;
              G[l0 * n3 + k0 * n2 + i0 * n1 + j0] = val;
              G[k0 * n3 + l0 * n2 + j0 * n1 + i0] = val;
              G[l0 * n3 + k0 * n2 + j0 * n1 + i0] = val;
            }
    }
  }
  free(pa);
  free(pb);
  free(sh);
  return nf;
}
