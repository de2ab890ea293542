// Molecular integrals on the GPU (McMurchie-Davidson, FP64): one-body S, T,
// V; (mu nu|la si) over shell quartets; Coulomb and exchange contractions of
// the stored (mu nu|la si) with a density; MO block extraction.
//
// Electron repulsion: one warp per shell quartet (bra pair P, ket pair Q).
// The warp walks the primitive quartets of P x Q 32 at a time: lane j
// evaluates the Boys function and the Hermite Coulomb integrals R_{tuv} of
// quartet j into its own shared-memory slab (prefactor folded in).  Classes
// with at most 9 Cartesian outputs (ss|ss, ps|ss, pp|ss, ps|ps, ds|ss), which
// carry the long contractions, contract each lane's quartet privately and sum
// over the warp at the end.  The others contract the 32 slabs one after the
// other, in two factored steps spread over the lanes:
//   Z[h1][cd]  = sum_h2 (-1)^|h2| E^{cd}_{h2} R[h1 + h2]
//   out[ab][cd] += sum_h1 E^{ab}_{h1} Z[h1][cd].
// The Cartesian block is then transformed to spherical d functions, scaled to
// unit-overlap functions and written in all eight permutations of
// (mu nu|la si).
//
// Boys function: F_{L+j}(T_k) tabulated at T_k = 0.05 k (k <= 800), a
// seven-term Taylor expansion in T - T_k (dF_n/dT = -F_{n+1}) for F_L and the
// downward recurrence F_n = (2T F_{n+1} + e^{-T}) / (2n + 1); above T = 40
// F_0 = (pi/T)^{1/2} / 2 and the upward recurrence.
#include "ints.h"

#include <cmath>
#include <cstring>

namespace gbcc {
namespace ints {

// ---------------------------------------------------------------------------
// host tables

const HermTables& herm_tables() {
  static const HermTables tab = [] {
    HermTables h;
    std::memset(&h, 0, sizeof(h));
    for (int t = 0; t <= kLtot; ++t)
      for (int u = 0; u <= kLtot; ++u)
        for (int v = 0; v <= kLtot; ++v) h.tuv[t][u][v] = -1;
    int n = 0;
    for (int m = 0; m <= kLtot; ++m)
      for (int t = m; t >= 0; --t)
        for (int u = m - t; u >= 0; --u) {
          const int v = m - t - u;
          h.t[n] = static_cast<int8_t>(t);
          h.u[n] = static_cast<int8_t>(u);
          h.v[n] = static_cast<int8_t>(v);
          h.tuv[t][u][v] = static_cast<int16_t>(n);
          ++n;
        }
    for (int k = 0; k < kNhMax; ++k) {
      const int t = h.t[k], u = h.u[k], v = h.v[k];
      h.i2[k] = -1;
      if (k == 0) continue;
      if (t > 0) {
        h.axis[k] = 0;
        h.i1[k] = static_cast<uint8_t>(h.tuv[t - 1][u][v]);
        if (t > 1) h.i2[k] = h.tuv[t - 2][u][v];
        h.c2[k] = static_cast<uint8_t>(t - 1);
      } else if (u > 0) {
        h.axis[k] = 1;
        h.i1[k] = static_cast<uint8_t>(h.tuv[t][u - 1][v]);
        if (u > 1) h.i2[k] = h.tuv[t][u - 2][v];
        h.c2[k] = static_cast<uint8_t>(u - 1);
      } else {
        h.axis[k] = 2;
        h.i1[k] = static_cast<uint8_t>(h.tuv[t][u][v - 1]);
        if (v > 1) h.i2[k] = h.tuv[t][u][v - 2];
        h.c2[k] = static_cast<uint8_t>(v - 1);
      }
    }
    for (int a = 0; a < kNhPair; ++a)
      for (int b = 0; b < kNhPair; ++b)
        h.sum[a][b] = static_cast<uint8_t>(h.tuv[h.t[a] + h.t[b]][h.u[a] + h.u[b]][h.v[a] + h.v[b]]);
    return h;
  }();
  return tab;
}

// F_n(T) = e^{-T} sum_k (2T)^k / ((2n+1)(2n+3)...(2n+2k+1)) for the highest
// order, the downward recurrence below it.
void boys_series(int nmax, double T, double* F) {
  const double e = std::exp(-T);
  double term = 1.0 / (2 * nmax + 1), sum = term;
  for (int k = 1; k < 1000; ++k) {
    term *= 2.0 * T / (2 * nmax + 2 * k + 1);
    sum += term;
    if (term < 1e-18 * sum) break;
  }
  F[nmax] = e * sum;
  for (int n = nmax - 1; n >= 0; --n) F[n] = (2.0 * T * F[n + 1] + e) / (2 * n + 1);
}

std::vector<double> boys_table() {
  std::vector<double> tab(static_cast<size_t>(kBoysPoints) * kBoysOrders);
  for (int k = 0; k < kBoysPoints; ++k) boys_series(kBoysOrders - 1, k * kBoysStep, &tab[k * kBoysOrders]);
  return tab;
}

// ---------------------------------------------------------------------------
// device building blocks

namespace {

constexpr double kPi = 3.14159265358979323846;

// tables a kernel keeps in shared memory
struct STab {
  int8_t axis[kNhMax];
  uint8_t i1[kNhMax];
  int16_t i2[kNhMax];
  uint8_t c2[kNhMax];
  uint8_t sum[kNhPair][kNhPair];
  int8_t t[kNhMax], u[kNhMax], v[kNhMax];
};

__device__ void load_tables(const HermTables* g, STab* s) {
  const int nt = blockDim.x;
  for (int k = threadIdx.x; k < kNhMax; k += nt) {
    s->axis[k] = g->axis[k];
    s->i1[k] = g->i1[k];
    s->i2[k] = g->i2[k];
    s->c2[k] = g->c2[k];
    s->t[k] = g->t[k];
    s->u[k] = g->u[k];
    s->v[k] = g->v[k];
  }
  for (int k = threadIdx.x; k < kNhPair * kNhPair; k += nt) (&s->sum[0][0])[k] = (&g->sum[0][0])[k];
}

__device__ __forceinline__ double inv_odd(int n) { return 1.0 / (2 * n + 1); }

// F_0..F_L(T)
__device__ __forceinline__ void boys_eval(int L, double T, const double* __restrict__ tab, double* F) {
  if (T < kBoysTmax) {
    const int k = __double2int_rn(T * (1.0 / kBoysStep));
    const double md = -(T - k * kBoysStep);
    const double* f = tab + k * kBoysOrders + L;
    double s = f[6];
    s = fma(s, md * (1.0 / 6.0), f[5]);
    s = fma(s, md * (1.0 / 5.0), f[4]);
    s = fma(s, md * (1.0 / 4.0), f[3]);
    s = fma(s, md * (1.0 / 3.0), f[2]);
    s = fma(s, md * (1.0 / 2.0), f[1]);
    s = fma(s, md, f[0]);
    F[L] = s;
    const double e = exp(-T);
    for (int n = L - 1; n >= 0; --n) F[n] = fma(2.0 * T, F[n + 1], e) * inv_odd(n);
  } else {
    const double e = exp(-T);
    F[0] = 0.5 * sqrt(kPi / T);
    const double h = 0.5 / T;
    for (int n = 0; n < L; ++n) F[n + 1] = ((2 * n + 1) * F[n] - e) * h;
  }
}

// R[h] = pref R^0_{tuv}(alpha, pq) for every (t,u,v) of degree <= L, in place:
// level n = L-1 .. 0 rewrites degrees L-n .. 1 from the level above (lower
// degrees are still of level n+1 when they are read), then R[0].
__device__ __forceinline__ void hermite_r(int L, double* R, double px, double py, double pz, double alpha,
                                          double pref, const double* __restrict__ boys, const STab& tab) {
  double F[kLtot + 1];
  boys_eval(L, alpha * (px * px + py * py + pz * pz), boys, F);
  double pw[kLtot + 1];
  pw[0] = pref;
  for (int n = 0; n < L; ++n) pw[n + 1] = pw[n] * (-2.0 * alpha);
  R[0] = pw[L] * F[L];
  for (int n = L - 1; n >= 0; --n) {
    const int hmax = nherm(L - n);
    for (int h = hmax - 1; h >= 1; --h) {
      const int ax = tab.axis[h];
      const double x = ax == 0 ? px : (ax == 1 ? py : pz);
      double val = x * R[tab.i1[h]];
      const int c = tab.c2[h];
      if (c) val = fma(static_cast<double>(c), R[tab.i2[h]], val);
      R[h] = val;
    }
    R[0] = pw[n] * F[n];
  }
}

__device__ __forceinline__ int nfunc(int l, int pure) { return (pure && l == 2) ? 5 : ncart(l); }

// Cartesian components of spherical function f of a shell (d: xy, yz,
// 2zz-xx-yy, xz, xx-yy over xx, xy, xz, yy, yz, zz); identity otherwise
__device__ __forceinline__ int sph_row(int l, int pure, int f, int* idx, double* c) {
  if (!(pure && l == 2)) {
    idx[0] = f;
    c[0] = 1.0;
    return 1;
  }
  switch (f) {
    case 0: idx[0] = 1; c[0] = 1.0; return 1;
    case 1: idx[0] = 4; c[0] = 1.0; return 1;
    case 2: idx[0] = 5; c[0] = 2.0; idx[1] = 0; c[1] = -1.0; idx[2] = 3; c[2] = -1.0; return 3;
    case 3: idx[0] = 2; c[0] = 1.0; return 1;
    default: idx[0] = 0; c[0] = 1.0; idx[1] = 3; c[1] = -1.0; return 2;
  }
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

struct EriKernelArgs {
  EriArgs a;
  const HermTables* herm;
};

template <int LA, int LB, int LC, int LD>
struct EriShape {
  static constexpr int NA = ncart(LA), NB = ncart(LB), NC = ncart(LC), ND = ncart(LD);
  static constexpr int NAB = NA * NB, NCD = NC * ND, NOUT = NAB * NCD;
  static constexpr int LAB = LA + LB, LCD = LC + LD, L = LAB + LCD;
  static constexpr int NHAB = nherm(LAB), NHCD = nherm(LCD), NR = nherm(L);
  static constexpr int NRP = NR | 1;  // odd slab stride: lanes hit distinct banks
  static constexpr bool PRIV = NOUT <= 9;
  static constexpr int NACC = PRIV ? NOUT : (NOUT + 31) / 32;
  static constexpr int ZSZ = PRIV ? 0 : NHAB * NCD;
  static constexpr int WARP_DBL = 32 * NRP + ZSZ;
  static_assert(NOUT <= 32 * NRP, "the Cartesian block reuses the R slabs");
};

template <int LA, int LB, int LC, int LD>
__global__ void __launch_bounds__(128) eri_kernel(EriKernelArgs ka) {
  using S = EriShape<LA, LB, LC, LD>;
  const EriArgs& a = ka.a;
  extern __shared__ double smem[];
  const int nwarps = blockDim.x >> 5;
  STab& tab = *reinterpret_cast<STab*>(smem + nwarps * S::WARP_DBL);
  load_tables(ka.herm, &tab);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t q = static_cast<int64_t>(blockIdx.x) * nwarps + warp;
  if (q >= a.nquart) return;
  int64_t ip, iq;
  if (a.same) {
    ip = static_cast<int64_t>((sqrt(8.0 * static_cast<double>(q) + 1.0) - 1.0) * 0.5);
    while (ip * (ip + 1) / 2 > q) --ip;
    while ((ip + 1) * (ip + 2) / 2 <= q) ++ip;
    iq = q - ip * (ip + 1) / 2;
  } else {
    ip = q / a.nq;
    iq = q % a.nq;
  }
  const PairInfo P = a.pairs[a.p0 + ip];
  const PairInfo Q = a.pairs[a.q0 + iq];
  double* Rs = smem + warp * S::WARP_DBL;
  double* Z = Rs + 32 * S::NRP;
  const double* Eab = a.E + P.e0;
  const double* Ecd = a.E + Q.e0;
  const int npq = Q.nprim;
  const int64_t nf = static_cast<int64_t>(P.nprim) * npq;
  double acc[S::NACC];
#pragma unroll
  for (int k = 0; k < S::NACC; ++k) acc[k] = 0.0;

  for (int64_t base = 0; base < nf; base += 32) {
    const int64_t f = base + lane;
    double* R = Rs + lane * S::NRP;
    if (f < nf) {
      const int kp = static_cast<int>(f / npq), kq = static_cast<int>(f % npq);
      const PrimPair pp = a.prim[P.prim0 + kp], qq = a.prim[Q.prim0 + kq];
      const double p = pp.p, qe = qq.p, spq = p + qe;
      const double alpha = p * qe / spq;
      const double pref = 2.0 * kPi * kPi * sqrt(kPi) / (p * qe * sqrt(spq));
      hermite_r(S::L, R, pp.px - qq.px, pp.py - qq.py, pp.pz - qq.pz, alpha, pref, a.boys, tab);
      if constexpr (S::PRIV) {
        const double* ea = Eab + static_cast<int64_t>(kp) * S::NAB * S::NHAB;
        const double* ec = Ecd + static_cast<int64_t>(kq) * S::NCD * S::NHCD;
#pragma unroll
        for (int ab = 0; ab < S::NAB; ++ab)
#pragma unroll
          for (int cd = 0; cd < S::NCD; ++cd) {
            double s = 0.0;
            for (int h1 = 0; h1 < S::NHAB; ++h1) {
              double z = 0.0;
              for (int h2 = 0; h2 < S::NHCD; ++h2) {
                const double e = ec[cd * S::NHCD + h2];
                const bool odd = (tab.t[h2] + tab.u[h2] + tab.v[h2]) & 1;
                z = fma(odd ? -e : e, R[tab.sum[h1][h2]], z);
              }
              s = fma(ea[ab * S::NHAB + h1], z, s);
            }
            acc[ab * S::NCD + cd] += s;
          }
      }
    }
    if constexpr (!S::PRIV) {
      __syncwarp();
      const int nvalid = static_cast<int>(nf - base < 32 ? nf - base : 32);
      for (int j = 0; j < nvalid; ++j) {
        const int64_t fj = base + j;
        const int kp = static_cast<int>(fj / npq), kq = static_cast<int>(fj % npq);
        const double* Rj = Rs + j * S::NRP;
        const double* ec = Ecd + static_cast<int64_t>(kq) * S::NCD * S::NHCD;
        for (int idx = lane; idx < S::NHAB * S::NCD; idx += 32) {
          const int h1 = idx / S::NCD, cd = idx % S::NCD;
          double z = 0.0;
          for (int h2 = 0; h2 < S::NHCD; ++h2) {
            const double e = ec[cd * S::NHCD + h2];
            const bool odd = (tab.t[h2] + tab.u[h2] + tab.v[h2]) & 1;
            z = fma(odd ? -e : e, Rj[tab.sum[h1][h2]], z);
          }
          Z[idx] = z;
        }
        __syncwarp();
        const double* ea = Eab + static_cast<int64_t>(kp) * S::NAB * S::NHAB;
#pragma unroll
        for (int k = 0; k < S::NACC; ++k) {
          const int o = lane + 32 * k;
          if (o < S::NOUT) {
            const int ab = o / S::NCD, cd = o % S::NCD;
            double s = 0.0;
            for (int h1 = 0; h1 < S::NHAB; ++h1) s = fma(ea[ab * S::NHAB + h1], Z[h1 * S::NCD + cd], s);
            acc[k] += s;
          }
        }
        __syncwarp();
      }
    }
  }
  __syncwarp();
  double* cart = Rs;  // the R slabs are free now
  if constexpr (S::PRIV) {
#pragma unroll
    for (int o = 0; o < S::NOUT; ++o) {
      const double v = warp_sum(acc[o]);
      if (lane == 0) cart[o] = v;
    }
  } else {
#pragma unroll
    for (int k = 0; k < S::NACC; ++k) {
      const int o = lane + 32 * k;
      if (o < S::NOUT) cart[o] = acc[k];
    }
  }
  __syncwarp();
  const int pure = a.pure;
  const int FA = nfunc(LA, pure), FB = nfunc(LB, pure), FC = nfunc(LC, pure), FD = nfunc(LD, pure);
  const int64_t n1 = a.nbf, n2 = n1 * n1, n3 = n2 * n1;
  for (int idx = lane; idx < FA * FB * FC * FD; idx += 32) {
    const int e4 = idx % FD, h3 = (idx / FD) % FC, g2 = (idx / (FD * FC)) % FB, f1 = idx / (FD * FC * FB);
    int ia[3], ib[3], ic[3], id[3];
    double ca[3], cb[3], cc[3], cd[3];
    const int na = sph_row(LA, pure, f1, ia, ca), nb = sph_row(LB, pure, g2, ib, cb);
    const int nc = sph_row(LC, pure, h3, ic, cc), nd = sph_row(LD, pure, e4, id, cd);
    double val = 0.0;
    for (int x = 0; x < na; ++x)
      for (int y = 0; y < nb; ++y)
        for (int z = 0; z < nc; ++z)
          for (int w = 0; w < nd; ++w)
            val += ca[x] * cb[y] * cc[z] * cd[w] * cart[((ia[x] * S::NB + ib[y]) * S::NC + ic[z]) * S::ND + id[w]];
    const int64_t i0 = P.f1 + f1, j0 = P.f2 + g2, k0 = Q.f1 + h3, l0 = Q.f2 + e4;
    val *= a.norm[i0] * a.norm[j0] * a.norm[k0] * a.norm[l0];
    double* G = a.G;
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

// device copy of the Hermite tables, one per device
const HermTables* device_tables() {
  static const HermTables* ptr[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return nullptr;
  if (!ptr[dev]) {
    void* p = nullptr;
    if (cudaMalloc(&p, sizeof(HermTables)) != cudaSuccess) return nullptr;
    cudaMemcpy(p, &herm_tables(), sizeof(HermTables), cudaMemcpyHostToDevice);
    ptr[dev] = static_cast<const HermTables*>(p);
  }
  return ptr[dev];
}

template <int LA, int LB, int LC, int LD>
void launch_eri_t(const EriArgs& a, cudaStream_t st) {
  using S = EriShape<LA, LB, LC, LD>;
  const size_t per_warp = S::WARP_DBL * sizeof(double);
  int warps = 4;
  while (warps > 1 && warps * per_warp + sizeof(STab) > 200 * 1024) --warps;
  const size_t bytes = warps * per_warp + sizeof(STab);
  static bool attr_set[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (bytes > 48 * 1024 && dev >= 0 && dev < 64 && !attr_set[dev]) {
    cudaFuncSetAttribute(eri_kernel<LA, LB, LC, LD>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         static_cast<int>(bytes));
    attr_set[dev] = true;
  }
  EriKernelArgs ka{a, device_tables()};
  const int64_t blocks = (a.nquart + warps - 1) / warps;
  eri_kernel<LA, LB, LC, LD><<<static_cast<unsigned>(blocks), 32 * warps, bytes, st>>>(ka);
}

// ---------------------------------------------------------------------------
// one-body integrals: one thread per Cartesian function pair

struct OneBodyKernelArgs {
  OneBodyArgs a;
  const HermTables* herm;
};

// E^{ia, j}_t for j <= jmax (fixed ia) along one axis: rows[j][t], t <= ia + j
__device__ void hermite_rows(int ia, int jmax, double ea, double eb, double xab, double rows[5][7]) {
  const double p = ea + eb, mu = ea * eb / p;
  const double xpa = -eb / p * xab, xpb = ea / p * xab, hp = 0.5 / p;
  double cur[7] = {0, 0, 0, 0, 0, 0, 0}, nxt[7];
  cur[0] = exp(-mu * xab * xab);
  for (int i = 1; i <= ia; ++i) {  // E^{i,0} from E^{i-1,0}
    for (int t = 0; t <= i; ++t) {
      double v = xpa * cur[t];
      if (t > 0) v += hp * cur[t - 1];
      if (t + 1 <= i - 1) v += (t + 1) * cur[t + 1];
      nxt[t] = v;
    }
    for (int t = 0; t <= i; ++t) cur[t] = nxt[t];
    for (int t = i + 1; t < 7; ++t) cur[t] = 0.0;
  }
  for (int t = 0; t < 7; ++t) rows[0][t] = cur[t];
  for (int j = 1; j <= jmax; ++j) {  // E^{ia,j} from E^{ia,j-1}
    const double* src = rows[j - 1];
    const int top = ia + j - 1;
    for (int t = 0; t < 7; ++t) {
      double v = 0.0;
      if (t <= top + 1) {
        v = xpb * (t <= top ? src[t] : 0.0);
        if (t > 0) v += hp * src[t - 1];
        if (t + 1 <= top) v += (t + 1) * src[t + 1];
      }
      rows[j][t] = v;
    }
  }
}

__global__ void __launch_bounds__(128) one_body_kernel(OneBodyKernelArgs ka) {
  const OneBodyArgs& a = ka.a;
  __shared__ STab tab;
  load_tables(ka.herm, &tab);
  __syncthreads();
  const int64_t n = a.ncart_total;
  const int64_t id = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (id >= n * n) return;
  const int mu = static_cast<int>(id / n), nu = static_cast<int>(id % n);
  const int sA = a.cf_shell[mu], sB = a.cf_shell[nu];
  const int cA = a.cf_comp[mu], cB = a.cf_comp[nu];
  const int ia[3] = {cA >> 4, (cA >> 2) & 3, cA & 3};
  const int ib[3] = {cB >> 4, (cB >> 2) & 3, cB & 3};
  const double A[3] = {a.sh_xyz[3 * sA], a.sh_xyz[3 * sA + 1], a.sh_xyz[3 * sA + 2]};
  const double B[3] = {a.sh_xyz[3 * sB], a.sh_xyz[3 * sB + 1], a.sh_xyz[3 * sB + 2]};
  double s = 0.0, t = 0.0, v = 0.0;
  double rows[3][5][7];
  double R[kNhPair];
  const int Lx = ia[0] + ib[0], Ly = ia[1] + ib[1], Lz = ia[2] + ib[2], L = Lx + Ly + Lz;
  for (int i = 0; i < a.sh_nprim[sA]; ++i) {
    const double ea = a.exps[a.sh_prim0[sA] + i];
    const double ca = a.coefs[a.sh_prim0[sA] + i];
    for (int j = 0; j < a.sh_nprim[sB]; ++j) {
      const double eb = a.exps[a.sh_prim0[sB] + j];
      const double cw = ca * a.coefs[a.sh_prim0[sB] + j];
      const double p = ea + eb;
      const double sq = sqrt(kPi / p);
      double s1[3], t1[3];
      for (int x = 0; x < 3; ++x) {
        hermite_rows(ia[x], ib[x] + 2, ea, eb, A[x] - B[x], rows[x]);
        const int jb = ib[x];
        s1[x] = rows[x][jb][0] * sq;
        double tv = -2.0 * eb * eb * rows[x][jb + 2][0] * sq + eb * (2 * jb + 1) * s1[x];
        if (jb >= 2) tv -= 0.5 * jb * (jb - 1) * rows[x][jb - 2][0] * sq;
        t1[x] = tv;
      }
      s += cw * s1[0] * s1[1] * s1[2];
      t += cw * (t1[0] * s1[1] * s1[2] + s1[0] * t1[1] * s1[2] + s1[0] * s1[1] * t1[2]);
      const double P[3] = {(ea * A[0] + eb * B[0]) / p, (ea * A[1] + eb * B[1]) / p, (ea * A[2] + eb * B[2]) / p};
      for (int c = 0; c < a.natom; ++c) {
        hermite_r(L, R, P[0] - a.atom_xyz[3 * c], P[1] - a.atom_xyz[3 * c + 1], P[2] - a.atom_xyz[3 * c + 2], p,
                  1.0, a.boys, tab);
        double h = 0.0;
        for (int tt = 0; tt <= Lx; ++tt)
          for (int uu = 0; uu <= Ly; ++uu)
            for (int vv = 0; vv <= Lz; ++vv) {
              // index of (tt,uu,vv): degree-major order
              const int m = tt + uu + vv;
              const int base = nherm(m - 1 < 0 ? -1 : m - 1);
              // within degree m: t descending, then u descending
              int off = 0;
              for (int t2 = m; t2 > tt; --t2) off += m - t2 + 1;
              off += (m - tt) - uu;
              h += rows[0][ib[0]][tt] * rows[1][ib[1]][uu] * rows[2][ib[2]][vv] * R[(m == 0 ? 0 : base) + off];
            }
        v -= a.zn[c] * cw * 2.0 * kPi / p * h;
      }
    }
  }
  a.S[id] = s;
  a.T[id] = t;
  a.V[id] = v;
}

// ---------------------------------------------------------------------------

__device__ __forceinline__ double block_sum(double v, double* sh) {
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0)
    for (int k = 0; k < static_cast<int>(blockDim.x >> 5); ++k) r += sh[k];
  __syncthreads();
  return r;
}

// one block per (mu, nu): J = sum G[mu nu la si] D[la si], K = sum G[mu la nu si] D[la si]
__global__ void __launch_bounds__(256) jk_kernel(int n, const double* __restrict__ G, const double* __restrict__ D,
                                                double* J, double* K) {
  __shared__ double sh[8];
  const int64_t nn = n;
  const int64_t mu = blockIdx.x / n, nu = blockIdx.x % n;
  const double* gj = G + (mu * nn + nu) * nn * nn;
  double sj = 0.0, sk = 0.0;
  for (int64_t x = threadIdx.x; x < nn * nn; x += blockDim.x) sj = fma(gj[x], D[x], sj);
  for (int64_t x = threadIdx.x; x < nn * nn; x += blockDim.x) {
    const int64_t la = x / nn, si = x % nn;
    sk = fma(G[((mu * nn + la) * nn + nu) * nn + si], D[x], sk);
  }
  sj = block_sum(sj, sh);
  sk = block_sum(sk, sh);
  if (threadIdx.x == 0) {
    J[mu * nn + nu] = sj;
    K[mu * nn + nu] = sk;
  }
}

struct Offsets4 {
  int64_t x, y, z, w;
};

__global__ void mo_block_kernel(int64_t n, const double* __restrict__ mo, int64_t d0, int64_t d1, int64_t d2,
                                int64_t d3, int4 perm, Offsets4 off, double* __restrict__ out) {
  const int64_t total = d0 * d1 * d2 * d3;
  for (int64_t idx = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; idx < total;
       idx += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    int64_t x[4];
    x[3] = idx % d3;
    x[2] = (idx / d3) % d2;
    x[1] = (idx / (d3 * d2)) % d1;
    x[0] = idx / (d3 * d2 * d1);
    const int64_t m0 = x[perm.x] + off.x, m1 = x[perm.y] + off.y, m2 = x[perm.z] + off.z, m3 = x[perm.w] + off.w;
    out[idx] = mo[((m0 * n + m1) * n + m2) * n + m3];
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// launchers

void launch_eri_class(int cP, int cQ, const EriArgs& a, cudaStream_t st) {
  if (a.nquart <= 0) return;
  // class index -> (l1, l2): 0 (0,0) 1 (1,0) 2 (1,1) 3 (2,0) 4 (2,1) 5 (2,2)
#define GBCC_ERI_CASE(P, Q, LA, LB, LC, LD) \
  if (cP == P && cQ == Q) return launch_eri_t<LA, LB, LC, LD>(a, st);
  GBCC_ERI_CASE(0, 0, 0, 0, 0, 0)
  GBCC_ERI_CASE(1, 0, 1, 0, 0, 0)
  GBCC_ERI_CASE(1, 1, 1, 0, 1, 0)
  GBCC_ERI_CASE(2, 0, 1, 1, 0, 0)
  GBCC_ERI_CASE(2, 1, 1, 1, 1, 0)
  GBCC_ERI_CASE(2, 2, 1, 1, 1, 1)
  GBCC_ERI_CASE(3, 0, 2, 0, 0, 0)
  GBCC_ERI_CASE(3, 1, 2, 0, 1, 0)
  GBCC_ERI_CASE(3, 2, 2, 0, 1, 1)
  GBCC_ERI_CASE(3, 3, 2, 0, 2, 0)
  GBCC_ERI_CASE(4, 0, 2, 1, 0, 0)
  GBCC_ERI_CASE(4, 1, 2, 1, 1, 0)
  GBCC_ERI_CASE(4, 2, 2, 1, 1, 1)
  GBCC_ERI_CASE(4, 3, 2, 1, 2, 0)
  GBCC_ERI_CASE(4, 4, 2, 1, 2, 1)
  GBCC_ERI_CASE(5, 0, 2, 2, 0, 0)
  GBCC_ERI_CASE(5, 1, 2, 2, 1, 0)
  GBCC_ERI_CASE(5, 2, 2, 2, 1, 1)
  GBCC_ERI_CASE(5, 3, 2, 2, 2, 0)
  GBCC_ERI_CASE(5, 4, 2, 2, 2, 1)
  GBCC_ERI_CASE(5, 5, 2, 2, 2, 2)
#undef GBCC_ERI_CASE
}

void launch_one_body(const OneBodyArgs& a, cudaStream_t st) {
  const int64_t n2 = static_cast<int64_t>(a.ncart_total) * a.ncart_total;
  if (n2 == 0) return;
  OneBodyKernelArgs ka{a, device_tables()};
  one_body_kernel<<<static_cast<unsigned>((n2 + 127) / 128), 128, 0, st>>>(ka);
}

void launch_coulomb_exchange(int n, const double* G, const double* D, double* J, double* K, cudaStream_t st) {
  if (n <= 0) return;
  jk_kernel<<<static_cast<unsigned>(n * n), 256, 0, st>>>(n, G, D, J, K);
}

void launch_mo_block(int64_t n, const double* mo, const int64_t dims[4], const int perm[4], const int64_t off[4],
                     double* out, cudaStream_t st) {
  const int64_t total = dims[0] * dims[1] * dims[2] * dims[3];
  if (total == 0) return;
  const int64_t blocks = std::min<int64_t>((total + 255) / 256, 152 * 64);
  mo_block_kernel<<<static_cast<unsigned>(blocks), 256, 0, st>>>(
      n, mo, dims[0], dims[1], dims[2], dims[3], make_int4(perm[0], perm[1], perm[2], perm[3]),
      Offsets4{off[0], off[1], off[2], off[3]}, out);
}

}  // namespace ints
}  // namespace gbcc
