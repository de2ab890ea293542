// C ABI of the SCF input producer (include/gbcc_scf.h): basis set-up, AO
// integrals on the device, closed-shell RHF and the AO -> MO transform into a
// CCSD handle.
//
// The RHF loop follows RHF::solve (src/mpqc/chemistry/qc/lcao/scf/
// rhf_impl.h:178-262): build F = H + 2J - K from the density, E = tr D (H + F)
// + E_nuc, the orbital gradient FDS - SDF, DIIS on F, new orbitals from the
// extrapolated F; stop when |dE| <= threshold and |FDS - SDF|_F / N^2 <=
// threshold.  D = C_occ C_occ^T, as the reference's density builder makes it.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/gbcc.h"
#include "../../include/gbcc_scf.h"
#include "engine.h"
#include "hostla.h"
#include "ints.h"
#include "kernels.h"

using gbcc::Error;
namespace I = gbcc::ints;

bool gbcc_internal_dims(const gbcc_handle* h, int64_t* o, int64_t* v, int* device);  // api.cpp

struct gbcc_scf {
  gbcc_scf_config cfg{};
  std::string last_error;
  cudaStream_t stream = nullptr;
  int nbf = 0, ncart = 0, nocc = 0, natom = 0, pure = 0;
  double e_nuc = 0.0;
  std::vector<double> S, H, X;   // normalised AO S, H; orthogonaliser S^{-1/2}
  std::vector<double> F, C, eps; // converged Fock (AO), orbitals, energies
  bool scf_done = false;
  double* d_G = nullptr;         // (mu nu|la si), nbf^4
  double* d_D = nullptr;
  double* d_J = nullptr;
  double* d_K = nullptr;
  double t_one = 0.0, t_eri = 0.0, t_scf = 0.0, t_tr = 0.0;
  int iters = 0;
  bool converged = false;
  double energy = 0.0;
};

namespace {

thread_local std::string g_scf_create_error;

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

template <class F>
gbcc_status scf_guarded(gbcc_scf* h, F&& f) {
  if (!h) return GBCC_ERR_INVALID_ARG;
  try {
    if (cudaSetDevice(h->cfg.device) != cudaSuccess) throw Error(GBCC_ERR_CUDA, "cudaSetDevice failed");
    const gbcc_status s = f();
    if (s == GBCC_OK) h->last_error.clear();
    return s;
  } catch (const Error& e) {
    cudaGetLastError();
    h->last_error = e.what();
    return e.status;
  } catch (const std::bad_alloc&) {
    h->last_error = "host allocation failed";
    return GBCC_ERR_OOM;
  } catch (const std::exception& e) {
    h->last_error = e.what();
    return GBCC_ERR_CUDA;
  }
}

// normalisation of a primitive x^l e^{-a r^2} component with (2l-1)!! in the denominator
double prim_norm(double a, int l) {
  double df = 1.0;
  for (int k = 2 * l - 1; k > 1; k -= 2) df *= k;
  return std::pow(2.0 * a / M_PI, 0.75) * std::pow(4.0 * a, 0.5 * l) / std::sqrt(df);
}

struct Shell {
  int l, atom, nprim, prim0, f0, c0;  // f0: first (spherical) function, c0: first Cartesian
  double xyz[3];
};

int nfunc(int l, int pure) { return (pure && l == 2) ? 5 : I::ncart(l); }

// rows of the spherical transform of one shell: T[f][c]
std::vector<double> sph_block(int l, int pure) {
  const int nc = I::ncart(l), nf = nfunc(l, pure);
  std::vector<double> T(nf * nc, 0.0);
  if (pure && l == 2) {
    const double rows[5][6] = {{0, 1, 0, 0, 0, 0}, {0, 0, 0, 0, 1, 0}, {-1, 0, 0, -1, 0, 2}, {0, 0, 1, 0, 0, 0},
                               {1, 0, 0, -1, 0, 0}};
    for (int f = 0; f < 5; ++f)
      for (int c = 0; c < 6; ++c) T[f * 6 + c] = rows[f][c];
  } else {
    for (int f = 0; f < nf; ++f) T[f * nc + f] = 1.0;
  }
  return T;
}

// E^{ij}_t along one axis (host), i <= la, j <= lb
void hermite_e_host(int la, int lb, double a, double b, double xab, double E[3][3][5]) {
  const double p = a + b, mu = a * b / p;
  const double xpa = -b / p * xab, xpb = a / p * xab, hp = 0.5 / p;
  std::memset(E, 0, sizeof(double) * 45);
  E[0][0][0] = std::exp(-mu * xab * xab);
  for (int i = 0; i <= la; ++i)
    for (int j = 0; j <= lb; ++j) {
      if (i == 0 && j == 0) continue;
      int ii, jj;
      double x;
      const double* src;
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

void comps(int l, int c[6][3]) {
  int n = 0;
  for (int i = l; i >= 0; --i)
    for (int j = l - i; j >= 0; --j) {
      c[n][0] = i;
      c[n][1] = j;
      c[n][2] = l - i - j;
      ++n;
    }
}

template <class T>
T* dev_upload(const std::vector<T>& v, cudaStream_t st) {
  if (v.empty()) return nullptr;
  T* p = static_cast<T*>(gbcc::dev_alloc(v.size() * sizeof(T)));
  GBCC_CK(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st));
  return p;
}

struct DevBuf {
  void* p = nullptr;
  DevBuf() = default;
  explicit DevBuf(size_t bytes) : p(gbcc::dev_alloc(bytes)) {}
  ~DevBuf() { gbcc::dev_free(p); }
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  template <class T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

// S, H and (mu nu|la si) of the molecule on the device
void build_integrals(gbcc_scf* h, const gbcc_molecule* mol, const gbcc_basis* bs) {
  cudaStream_t st = h->stream;
  const int ns = bs->nshell;
  std::vector<Shell> sh(ns);
  std::vector<double> exps, coefs;
  int f = 0, c = 0, p0 = 0;
  for (int s = 0; s < ns; ++s) {
    Shell& x = sh[s];
    x.l = bs->l[s];
    x.atom = bs->atom[s];
    x.nprim = bs->nprim[s];
    x.prim0 = p0;
    x.f0 = f;
    x.c0 = c;
    for (int k = 0; k < 3; ++k) x.xyz[k] = mol->xyz[3 * x.atom + k];
    for (int i = 0; i < x.nprim; ++i) {
      const double a = bs->exps[p0 + i];
      exps.push_back(a);
      coefs.push_back(bs->coefs[p0 + i] * prim_norm(a, x.l));
    }
    p0 += x.nprim;
    f += nfunc(x.l, h->pure);
    c += I::ncart(x.l);
  }
  h->nbf = f;
  h->ncart = c;
  const int N = f, NC = c;

  // ---- one-body integrals (Cartesian, unnormalised) on the device
  const double t0 = now_s();
  std::vector<int> cf_shell(NC), cf_comp(NC), sh_nprim(ns), sh_prim0(ns);
  std::vector<double> sh_xyz(3 * ns), zn(h->natom), axyz(mol->xyz, mol->xyz + 3 * h->natom);
  for (int a = 0; a < h->natom; ++a) zn[a] = mol->charge[a];
  for (int s = 0; s < ns; ++s) {
    int cc[6][3];
    comps(sh[s].l, cc);
    for (int k = 0; k < I::ncart(sh[s].l); ++k) {
      cf_shell[sh[s].c0 + k] = s;
      cf_comp[sh[s].c0 + k] = cc[k][0] * 16 + cc[k][1] * 4 + cc[k][2];
    }
    sh_nprim[s] = sh[s].nprim;
    sh_prim0[s] = sh[s].prim0;
    for (int k = 0; k < 3; ++k) sh_xyz[3 * s + k] = sh[s].xyz[k];
  }
  const std::vector<double> boys = I::boys_table();
  double* d_boys = dev_upload(boys, st);
  struct Frees {
    std::vector<void*> p;
    ~Frees() {
      for (void* q : p) gbcc::dev_free(q);
    }
  } frees;
  frees.p.push_back(d_boys);
  auto up = [&](auto& v) {
    auto* q = dev_upload(v, st);
    frees.p.push_back(q);
    return q;
  };
  I::OneBodyArgs ob{};
  ob.ncart_total = NC;
  ob.cf_shell = up(cf_shell);
  ob.cf_comp = up(cf_comp);
  ob.sh_nprim = up(sh_nprim);
  ob.sh_prim0 = up(sh_prim0);
  ob.sh_xyz = up(sh_xyz);
  ob.exps = up(exps);
  ob.coefs = up(coefs);
  ob.natom = h->natom;
  ob.zn = up(zn);
  ob.atom_xyz = up(axyz);
  ob.boys = d_boys;
  DevBuf dS(sizeof(double) * NC * NC), dT(sizeof(double) * NC * NC), dV(sizeof(double) * NC * NC);
  ob.S = dS.as<double>();
  ob.T = dT.as<double>();
  ob.V = dV.as<double>();
  I::launch_one_body(ob, st);
  GBCC_CK(cudaGetLastError());
  std::vector<double> Sc(NC * NC), Tc(NC * NC), Vc(NC * NC);
  GBCC_CK(cudaMemcpyAsync(Sc.data(), ob.S, sizeof(double) * NC * NC, cudaMemcpyDeviceToHost, st));
  GBCC_CK(cudaMemcpyAsync(Tc.data(), ob.T, sizeof(double) * NC * NC, cudaMemcpyDeviceToHost, st));
  GBCC_CK(cudaMemcpyAsync(Vc.data(), ob.V, sizeof(double) * NC * NC, cudaMemcpyDeviceToHost, st));
  GBCC_CK(cudaStreamSynchronize(st));
  // spherical transform Tm (N x NC, block diagonal) and unit-overlap scaling
  std::vector<double> Tm(static_cast<size_t>(N) * NC, 0.0);
  for (int s = 0; s < ns; ++s) {
    const auto blk = sph_block(sh[s].l, h->pure);
    const int nf = nfunc(sh[s].l, h->pure), nc = I::ncart(sh[s].l);
    for (int a = 0; a < nf; ++a)
      for (int b = 0; b < nc; ++b) Tm[static_cast<size_t>(sh[s].f0 + a) * NC + sh[s].c0 + b] = blk[a * nc + b];
  }
  auto sandwich = [&](const std::vector<double>& M) {  // Tm M Tm^T
    std::vector<double> tmp(static_cast<size_t>(N) * NC, 0.0), out(static_cast<size_t>(N) * N, 0.0);
    gbcc::hostla::gemm_nn(N, NC, NC, Tm.data(), M.data(), tmp.data());
    gbcc::hostla::gemm_nt(N, N, NC, tmp.data(), Tm.data(), out.data());
    return out;
  };
  std::vector<double> S = sandwich(Sc), Hm = sandwich(Tc);
  const std::vector<double> Vs = sandwich(Vc);
  std::vector<double> norm(N);
  for (int i = 0; i < N; ++i) {
    const double d = S[static_cast<size_t>(i) * N + i];
    if (!(d > 0.0)) throw Error(GBCC_ERR_INVALID_ARG, "basis function with non-positive self-overlap");
    norm[i] = 1.0 / std::sqrt(d);
  }
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) {
      const size_t k = static_cast<size_t>(i) * N + j;
      S[k] *= norm[i] * norm[j];
      Hm[k] = (Hm[k] + Vs[k]) * norm[i] * norm[j];
    }
  h->S = std::move(S);
  h->H = std::move(Hm);
  h->t_one = now_s() - t0;

  // ---- shell pairs (first shell with the larger l), sorted by class
  const double t1 = now_s();
  struct PairTmp {
    int cls;
    I::PairInfo info;
    std::vector<I::PrimPair> prim;
    std::vector<double> E;
  };
  std::vector<std::vector<PairTmp>> bycls(I::kNumPairClasses);
  const auto& herm = I::herm_tables();
  for (int a = 0; a < ns; ++a)
    for (int b = 0; b <= a; ++b) {
      int s1 = a, s2 = b;
      if (sh[s1].l < sh[s2].l) std::swap(s1, s2);
      const Shell &A = sh[s1], &B = sh[s2];
      PairTmp pt;
      pt.cls = I::pair_class(A.l, B.l);
      pt.info = I::PairInfo{s1, s2, A.l, B.l, A.f0, B.f0, A.nprim * B.nprim, 0, 0};
      int ca[6][3], cb[6][3];
      comps(A.l, ca);
      comps(B.l, cb);
      const int na = I::ncart(A.l), nb = I::ncart(B.l), nh = I::nherm(A.l + B.l);
      for (int i = 0; i < A.nprim; ++i)
        for (int j = 0; j < B.nprim; ++j) {
          const double ea = exps[A.prim0 + i], eb = exps[B.prim0 + j], p = ea + eb;
          const double cw = coefs[A.prim0 + i] * coefs[B.prim0 + j];
          double E[3][3][3][5];
          for (int x = 0; x < 3; ++x) hermite_e_host(A.l, B.l, ea, eb, A.xyz[x] - B.xyz[x], E[x]);
          pt.prim.push_back(I::PrimPair{p, (ea * A.xyz[0] + eb * B.xyz[0]) / p, (ea * A.xyz[1] + eb * B.xyz[1]) / p,
                                        (ea * A.xyz[2] + eb * B.xyz[2]) / p});
          for (int x = 0; x < na; ++x)
            for (int y = 0; y < nb; ++y)
              for (int k = 0; k < nh; ++k) {
                const int t = herm.t[k], u = herm.u[k], v = herm.v[k];
                const int* i3 = ca[x];
                const int* j3 = cb[y];
                double val = 0.0;
                if (t <= i3[0] + j3[0] && u <= i3[1] + j3[1] && v <= i3[2] + j3[2])
                  val = cw * E[0][i3[0]][j3[0]][t] * E[1][i3[1]][j3[1]][u] * E[2][i3[2]][j3[2]][v];
                pt.E.push_back(val);
              }
        }
      bycls[pt.cls].push_back(std::move(pt));
    }
  std::vector<I::PairInfo> pairs;
  std::vector<I::PrimPair> prim;
  std::vector<double> Edat;
  std::vector<int> cls_start(I::kNumPairClasses + 1, 0);
  for (int k = 0; k < I::kNumPairClasses; ++k) {
    cls_start[k] = static_cast<int>(pairs.size());
    for (auto& pt : bycls[k]) {
      pt.info.prim0 = static_cast<int>(prim.size());
      pt.info.e0 = static_cast<int64_t>(Edat.size());
      pairs.push_back(pt.info);
      prim.insert(prim.end(), pt.prim.begin(), pt.prim.end());
      Edat.insert(Edat.end(), pt.E.begin(), pt.E.end());
    }
  }
  cls_start[I::kNumPairClasses] = static_cast<int>(pairs.size());
  bycls.clear();

  const size_t n4 = static_cast<size_t>(N) * N * N * N;
  h->d_G = static_cast<double*>(gbcc::dev_alloc(n4 * sizeof(double)));
  GBCC_CK(cudaMemsetAsync(h->d_G, 0, n4 * sizeof(double), st));
  I::EriArgs ea{};
  ea.pairs = up(pairs);
  ea.prim = up(prim);
  ea.E = up(Edat);
  ea.boys = d_boys;
  ea.norm = up(norm);
  ea.nbf = N;
  ea.pure = h->pure;
  ea.G = h->d_G;
  for (int cp = 0; cp < I::kNumPairClasses; ++cp)
    for (int cq = 0; cq <= cp; ++cq) {
      ea.p0 = cls_start[cp];
      ea.np = cls_start[cp + 1] - cls_start[cp];
      ea.q0 = cls_start[cq];
      ea.nq = cls_start[cq + 1] - cls_start[cq];
      ea.same = cp == cq;
      ea.nquart = ea.same ? static_cast<int64_t>(ea.np) * (ea.np + 1) / 2 : static_cast<int64_t>(ea.np) * ea.nq;
      I::launch_eri_class(cp, cq, ea, st);
      GBCC_CK(cudaGetLastError());
    }
  GBCC_CK(cudaStreamSynchronize(st));
  h->t_eri = now_s() - t1;
}

// orbitals of Fock matrix F: eigenvectors of X^T F X, C = X C'
void diagonalise_fock(const gbcc_scf* h, const std::vector<double>& F, std::vector<double>& C,
                      std::vector<double>& eps) {
  const int N = h->nbf;
  std::vector<double> tmp(static_cast<size_t>(N) * N), Fp(static_cast<size_t>(N) * N), V;
  gbcc::hostla::gemm_tn(N, N, N, h->X.data(), F.data(), tmp.data());   // X^T F
  gbcc::hostla::gemm_nn(N, N, N, tmp.data(), h->X.data(), Fp.data());  // X^T F X
  gbcc::hostla::symmetrize(N, Fp.data());
  gbcc::hostla::eigh(N, Fp, eps, V);
  C.assign(static_cast<size_t>(N) * N, 0.0);
  gbcc::hostla::gemm_nn(N, N, N, h->X.data(), V.data(), C.data());
}

void density(int N, int nocc, const std::vector<double>& C, std::vector<double>& D) {
  D.assign(static_cast<size_t>(N) * N, 0.0);
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) {
      double s = 0.0;
      for (int k = 0; k < nocc; ++k) s += C[static_cast<size_t>(i) * N + k] * C[static_cast<size_t>(j) * N + k];
      D[static_cast<size_t>(i) * N + j] = s;
    }
}

// rows x K panel times C: dst[cm[r] + cn[s]] = sum_k src[r K + k] C[k][s], in row chunks
void quarter(const double* src, int64_t rows, int64_t K, const double* d_Ct, int64_t n, const std::vector<int64_t>& cm,
             const std::vector<int64_t>& cn, double* dst, cudaStream_t st) {
  DevBuf dcm(cm.size() * sizeof(int64_t)), dcn(cn.size() * sizeof(int64_t));
  GBCC_CK(cudaMemcpyAsync(dcm.p, cm.data(), cm.size() * sizeof(int64_t), cudaMemcpyHostToDevice, st));
  GBCC_CK(cudaMemcpyAsync(dcn.p, cn.data(), cn.size() * sizeof(int64_t), cudaMemcpyHostToDevice, st));
  const int64_t chunk = 4000000;  // rows per launch (64-row tiles: grid.y < 65536)
  for (int64_t r0 = 0; r0 < rows; r0 += chunk) {
    gbcc::GemmF64Args g{};
    g.M = std::min(chunk, rows - r0);
    g.N = n;
    g.K = K;
    g.ksplit = 1;
    g.A = src + r0 * K;
    g.lda = K;
    g.B = d_Ct;
    g.ldb = K;
    g.C = dst;
    g.cm = dcm.as<int64_t>() + r0;
    g.cn = dcn.as<int64_t>();
    g.alpha = 1.0;
    g.beta = 0.0;
    gbcc::launch_gemm_f64(g, st);
    GBCC_CK(cudaGetLastError());
  }
  GBCC_CK(cudaStreamSynchronize(st));  // the offset tables are freed on return
}

}  // namespace

extern "C" {

void gbcc_scf_config_default(gbcc_scf_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->device = 0;
  c->max_iter = 30;
  c->threshold = 1e-11;
  c->n_diis = 8;
  c->verbose = 0;
}

gbcc_status gbcc_scf_create(gbcc_scf** out, const gbcc_molecule* mol, const gbcc_basis* bs,
                            const gbcc_scf_config* cfg) {
  g_scf_create_error.clear();
  if (!out || !mol || !bs || !cfg) {
    g_scf_create_error = "gbcc_scf_create: NULL argument";
    return GBCC_ERR_INVALID_ARG;
  }
  *out = nullptr;
  auto h = std::make_unique<gbcc_scf>();
  h->cfg = *cfg;
  try {
    if (mol->natom < 1 || !mol->charge || !mol->xyz) throw Error(GBCC_ERR_INVALID_ARG, "empty molecule");
    if (bs->nshell < 1 || !bs->atom || !bs->l || !bs->nprim || !bs->exps || !bs->coefs)
      throw Error(GBCC_ERR_INVALID_ARG, "empty basis");
    if (cfg->max_iter < 1 || !(cfg->threshold > 0.0) || cfg->n_diis < 1 || cfg->n_diis > 32)
      throw Error(GBCC_ERR_INVALID_ARG, "bad SCF configuration");
    double zsum = 0.0;
    for (int a = 0; a < mol->natom; ++a) {
      const double z = mol->charge[a];
      if (!(z >= 0.0) || z != std::floor(z) || z > 118)
        throw Error(GBCC_ERR_INVALID_ARG, "nuclear charges must be integers in 0..118");
      for (int k = 0; k < 3; ++k)
        if (!std::isfinite(mol->xyz[3 * a + k])) throw Error(GBCC_ERR_INVALID_ARG, "non-finite coordinate");
      zsum += z;
    }
    const double nel = zsum - mol->mol_charge;
    if (nel < 2 || std::fmod(nel, 2.0) != 0.0)
      throw Error(GBCC_ERR_INVALID_ARG, "closed-shell RHF needs an even, positive electron count");
    int64_t nprim_total = 0;
    for (int s = 0; s < bs->nshell; ++s) {
      if (bs->l[s] < 0 || bs->l[s] > I::kLmax) throw Error(GBCC_ERR_INVALID_ARG, "shells up to l = 2 (d) only");
      if (bs->atom[s] < 0 || bs->atom[s] >= mol->natom) throw Error(GBCC_ERR_INVALID_ARG, "shell atom out of range");
      if (bs->nprim[s] < 1 || bs->nprim[s] > 64) throw Error(GBCC_ERR_INVALID_ARG, "1..64 primitives per shell");
      for (int i = 0; i < bs->nprim[s]; ++i) {
        const double a = bs->exps[nprim_total + i], c = bs->coefs[nprim_total + i];
        if (!(a > 0.0) || !std::isfinite(a) || !std::isfinite(c))
          throw Error(GBCC_ERR_INVALID_ARG, "exponents must be positive and coefficients finite");
      }
      nprim_total += bs->nprim[s];
    }
    h->natom = mol->natom;
    h->pure = bs->pure ? 1 : 0;
    h->nocc = static_cast<int>(nel / 2);
    for (int a = 0; a < mol->natom; ++a)
      for (int b = 0; b < a; ++b) {
        double r2 = 0.0;
        for (int k = 0; k < 3; ++k) {
          const double d = mol->xyz[3 * a + k] - mol->xyz[3 * b + k];
          r2 += d * d;
        }
        if (!(r2 > 1e-8)) throw Error(GBCC_ERR_INVALID_ARG, "two nuclei at the same position");
        h->e_nuc += mol->charge[a] * mol->charge[b] / std::sqrt(r2);
      }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
      cudaGetLastError();
      throw Error(GBCC_ERR_CUDA, "no CUDA device available");
    }
    if (cfg->device < 0 || cfg->device >= ndev) throw Error(GBCC_ERR_INVALID_ARG, "bad device ordinal");
    GBCC_CK(cudaSetDevice(cfg->device));
    GBCC_CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    build_integrals(h.get(), mol, bs);
    if (h->nocc > h->nbf) throw Error(GBCC_ERR_INVALID_ARG, "more occupied orbitals than basis functions");
    // symmetric orthogonaliser X = S^{-1/2}
    const int N = h->nbf;
    std::vector<double> w, U, Sc = h->S;
    gbcc::hostla::eigh(N, Sc, w, U);
    if (!(w[0] > 1e-10)) throw Error(GBCC_ERR_INVALID_ARG, "overlap matrix (near) singular");
    h->X.assign(static_cast<size_t>(N) * N, 0.0);
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j) {
        double s = 0.0;
        for (int k = 0; k < N; ++k)
          s += U[static_cast<size_t>(i) * N + k] * U[static_cast<size_t>(j) * N + k] / std::sqrt(w[k]);
        h->X[static_cast<size_t>(i) * N + j] = s;
      }
    h->d_D = static_cast<double*>(gbcc::dev_alloc(sizeof(double) * N * N));
    h->d_J = static_cast<double*>(gbcc::dev_alloc(sizeof(double) * N * N));
    h->d_K = static_cast<double*>(gbcc::dev_alloc(sizeof(double) * N * N));
  } catch (const Error& e) {
    g_scf_create_error = e.what();
    gbcc_scf_destroy(h.release());
    return e.status;
  } catch (const std::exception& e) {
    g_scf_create_error = e.what();
    gbcc_scf_destroy(h.release());
    return GBCC_ERR_CUDA;
  }
  *out = h.release();
  return GBCC_OK;
}

gbcc_status gbcc_scf_run(gbcc_scf* h, gbcc_scf_report* report) {
  return scf_guarded(h, [&]() -> gbcc_status {
    const int N = h->nbf, nocc = h->nocc;
    const size_t NN = static_cast<size_t>(N) * N;
    const double t0 = now_s();
    std::vector<double> C, eps, D, J(NN), K(NN), F(NN), FDS(NN), SDF(NN), tmp(NN), tmp2(NN);
    diagonalise_fock(h, h->H, C, eps);  // core-Hamiltonian guess
    density(N, nocc, C, D);
    std::vector<std::vector<double>> fs, gs;
    const double thr = h->cfg.threshold;
    double e_old = 0.0, de = 1.0, grad = 1.0;
    bool conv = false;
    int it = 0;
    if (h->cfg.verbose) std::printf("Starting SCF:\n\tThreshold: %g\n\tMaximum number of iterations: %d\n", thr, h->cfg.max_iter);
    while (it < h->cfg.max_iter) {
      GBCC_CK(cudaMemcpyAsync(h->d_D, D.data(), NN * sizeof(double), cudaMemcpyHostToDevice, h->stream));
      gbcc::ints::launch_coulomb_exchange(N, h->d_G, h->d_D, h->d_J, h->d_K, h->stream);
      GBCC_CK(cudaGetLastError());
      GBCC_CK(cudaMemcpyAsync(J.data(), h->d_J, NN * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
      GBCC_CK(cudaMemcpyAsync(K.data(), h->d_K, NN * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
      GBCC_CK(cudaStreamSynchronize(h->stream));
      double e = h->e_nuc;
      for (size_t k = 0; k < NN; ++k) {
        F[k] = h->H[k] + 2.0 * J[k] - K[k];
        e += D[k] * (h->H[k] + F[k]);
      }
      gbcc::hostla::symmetrize(N, F.data());
      // orbital gradient FDS - SDF
      gbcc::hostla::gemm_nn(N, N, N, F.data(), D.data(), tmp.data());
      gbcc::hostla::gemm_nn(N, N, N, tmp.data(), h->S.data(), FDS.data());
      gbcc::hostla::gemm_nn(N, N, N, h->S.data(), D.data(), tmp2.data());
      gbcc::hostla::gemm_nn(N, N, N, tmp2.data(), F.data(), SDF.data());
      double g2 = 0.0;
      std::vector<double> G(NN);
      for (size_t k = 0; k < NN; ++k) {
        G[k] = FDS[k] - SDF[k];
        g2 += G[k] * G[k];
      }
      grad = std::sqrt(g2) / static_cast<double>(NN);
      de = std::fabs(e - e_old);
      e_old = e;
      ++it;
      if (h->cfg.verbose)
        std::printf("iteration: %d\n\tEnergy: %.15f\n\tabs(Energy Change): %.3e\n\t(Gradient Norm)/n^2: %.3e\n", it, e,
                    de, grad);
      if (!std::isfinite(e)) throw Error(GBCC_ERR_NUMERIC, "non-finite SCF energy");
      h->F = F;
      h->energy = e;
      if (it > 1 && de <= thr && grad <= thr) {
        conv = true;
        break;
      }
      // DIIS on F with the gradient (Pulay)
      fs.push_back(F);
      gs.push_back(G);
      if (static_cast<int>(fs.size()) > h->cfg.n_diis) {
        fs.erase(fs.begin());
        gs.erase(gs.begin());
      }
      const int m = static_cast<int>(fs.size());
      std::vector<double> B((m + 1) * (m + 1), -1.0), rhs(m + 1, 0.0);
      B[m * (m + 1) + m] = 0.0;
      rhs[m] = -1.0;
      for (int i = 0; i < m; ++i)
        for (int j = 0; j <= i; ++j) {
          double s = 0.0;
          for (size_t k = 0; k < NN; ++k) s += gs[i][k] * gs[j][k];
          B[i * (m + 1) + j] = B[j * (m + 1) + i] = s;
        }
      std::vector<double> coef;
      std::vector<double> Fd(NN, 0.0);
      if (gbcc::hostla::solve(m + 1, B, rhs, coef)) {
        for (int i = 0; i < m; ++i)
          for (size_t k = 0; k < NN; ++k) Fd[k] += coef[i] * fs[i][k];
      } else {
        Fd = F;
      }
      diagonalise_fock(h, Fd, C, eps);
      density(N, nocc, C, D);
    }
    // canonical orbitals of the last Fock matrix
    diagonalise_fock(h, h->F, h->C, h->eps);
    h->scf_done = true;
    h->iters = it;
    h->converged = conv;
    h->t_scf = now_s() - t0;
    if (report) {
      std::memset(report, 0, sizeof(*report));
      report->nbf = N;
      report->nocc = nocc;
      report->iters = it;
      report->converged = conv ? 1 : 0;
      report->energy = h->energy;
      report->e_nuc = h->e_nuc;
      report->seconds_one_body = h->t_one;
      report->seconds_eri = h->t_eri;
      report->seconds_scf = h->t_scf;
      report->seconds_transform = h->t_tr;
    }
    if (!conv) {
      h->last_error = "RHF SCF did not converge";
      return GBCC_ERR_NOT_CONVERGED;
    }
    return GBCC_OK;
  });
}

gbcc_status gbcc_scf_ao(gbcc_scf* h, double* S, double* H, double* G) {
  return scf_guarded(h, [&]() -> gbcc_status {
    const size_t NN = static_cast<size_t>(h->nbf) * h->nbf;
    if (S) std::memcpy(S, h->S.data(), NN * sizeof(double));
    if (H) std::memcpy(H, h->H.data(), NN * sizeof(double));
    if (G) {
      GBCC_CK(cudaMemcpyAsync(G, h->d_G, NN * NN * sizeof(double), cudaMemcpyDefault, h->stream));
      GBCC_CK(cudaStreamSynchronize(h->stream));
    }
    return GBCC_OK;
  });
}

gbcc_status gbcc_scf_orbitals(gbcc_scf* h, double* C, double* eps) {
  return scf_guarded(h, [&]() -> gbcc_status {
    if (!h->scf_done) throw Error(GBCC_ERR_STATE, "gbcc_scf_orbitals: run the SCF first");
    const size_t N = h->nbf;
    if (C) std::memcpy(C, h->C.data(), N * N * sizeof(double));
    if (eps) std::memcpy(eps, h->eps.data(), N * sizeof(double));
    return GBCC_OK;
  });
}

gbcc_status gbcc_scf_ccsd_inputs(gbcc_scf* h, int32_t n_frozen, gbcc_handle* cc) {
  return scf_guarded(h, [&]() -> gbcc_status {
    if (!h->scf_done) throw Error(GBCC_ERR_STATE, "gbcc_scf_ccsd_inputs: run the SCF first");
    if (!cc) throw Error(GBCC_ERR_INVALID_ARG, "gbcc_scf_ccsd_inputs: NULL CCSD handle");
    int64_t o = 0, v = 0;
    int dev = -1;
    if (!gbcc_internal_dims(cc, &o, &v, &dev)) throw Error(GBCC_ERR_INVALID_ARG, "bad CCSD handle");
    const int N = h->nbf, nocc = h->nocc;
    if (n_frozen < 0 || n_frozen >= nocc) throw Error(GBCC_ERR_INVALID_ARG, "n_frozen out of range");
    if (o != nocc - n_frozen || v != N - nocc)
      throw Error(GBCC_ERR_INVALID_ARG, "CCSD handle dimensions do not match: need o = " +
                                            std::to_string(nocc - n_frozen) + ", v = " + std::to_string(N - nocc));
    if (dev != h->cfg.device) throw Error(GBCC_ERR_INVALID_ARG, "CCSD handle is on another device");
    const double t0 = now_s();
    cudaStream_t st = h->stream;
    const int64_t n = N, N3 = n * n * n;
    // C^T (n x N): Ct[s][sigma] = C[sigma][s]
    std::vector<double> Ct(static_cast<size_t>(n) * N);
    for (int s = 0; s < n; ++s)
      for (int k = 0; k < N; ++k) Ct[static_cast<size_t>(s) * N + k] = h->C[static_cast<size_t>(k) * N + s];
    DevBuf dCt(Ct.size() * sizeof(double));
    GBCC_CK(cudaMemcpyAsync(dCt.p, Ct.data(), Ct.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    DevBuf A(sizeof(double) * n * N3), B(sizeof(double) * n * N3);
    std::vector<int64_t> cm, cn(n);
    // Q1: X1[mu nu][s][la] = sum_si G[mu nu la si] C[si][s]
    cm.resize(N3);
    for (int64_t r = 0; r < N3; ++r) cm[r] = (r / N) * (n * N) + (r % N);
    for (int64_t s = 0; s < n; ++s) cn[s] = s * N;
    quarter(h->d_G, N3, N, dCt.as<double>(), n, cm, cn, A.as<double>(), st);
    // Q2: X2[s][r][mu][nu] = sum_la X1[mu nu][s][la] C[la][r]; rows (mu nu, s)
    cm.resize(static_cast<size_t>(n) * N * N);
    for (int64_t r = 0; r < n * N * N; ++r) {
      const int64_t munu = r / n, s = r % n;
      cm[r] = s * (n * N * N) + munu;
    }
    for (int64_t q = 0; q < n; ++q) cn[q] = q * N * N;
    quarter(A.as<double>(), n * N * N, N, dCt.as<double>(), n, cm, cn, B.as<double>(), st);
    // Q3: X3[s][r][q][mu] = sum_nu X2[s][r][mu][nu] C[nu][q]; rows (s r, mu)
    cm.resize(static_cast<size_t>(n) * n * N);
    for (int64_t r = 0; r < n * n * N; ++r) cm[r] = (r / N) * (n * N) + (r % N);
    for (int64_t q = 0; q < n; ++q) cn[q] = q * N;
    quarter(B.as<double>(), n * n * N, N, dCt.as<double>(), n, cm, cn, A.as<double>(), st);
    // Q4: mo[p][q][r][s] = sum_mu X3[s][r][q][mu] C[mu][p]; rows (s r q)
    cm.resize(static_cast<size_t>(n) * n * n);
    for (int64_t r = 0; r < n * n * n; ++r) {
      const int64_t s = r / (n * n), rr = (r / n) % n, q = r % n;
      cm[r] = q * n * n + rr * n + s;
    }
    for (int64_t p = 0; p < n; ++p) cn[p] = p * n * n * n;
    quarter(A.as<double>(), n * n * n, N, dCt.as<double>(), n, cm, cn, B.as<double>(), st);
    std::vector<int64_t>().swap(cm);
    const double* mo = B.as<double>();

    gbcc_inputs in{};
    const gbcc_status ds = gbcc_device_inputs(cc, &in);
    if (ds != GBCC_OK) throw Error(ds, std::string("gbcc_device_inputs: ") + gbcc_last_error(cc));
    GBCC_CK(cudaSetDevice(h->cfg.device));
    const int64_t fz = n_frozen, no = nocc;
    struct Blk {
      double* out;
      int64_t d[4];
      int64_t off[4];  // per MO index (chemists' (pq|rs) order)
    };
    const int perm[4] = {0, 2, 1, 3};  // <pq|rs> = (pr|qs)
    const Blk blocks[] = {
        {const_cast<double*>(in.Gijab), {o, o, v, v}, {fz, no, fz, no}},
        {const_cast<double*>(in.Gijkl), {o, o, o, o}, {fz, fz, fz, fz}},
        {const_cast<double*>(in.Giajb), {o, v, o, v}, {fz, fz, no, no}},
        {const_cast<double*>(in.Gijka), {o, o, o, v}, {fz, fz, fz, no}},
        {const_cast<double*>(in.Giabc), {o, v, v, v}, {fz, no, no, no}},
        {const_cast<double*>(in.Gabcd), {v, v, v, v}, {no, no, no, no}},
    };
    for (const Blk& b : blocks) {
      gbcc::ints::launch_mo_block(n, mo, b.d, perm, b.off, b.out, st);
      GBCC_CK(cudaGetLastError());
    }
    // Fock blocks and orbital energies: Fmo = C^T F C
    std::vector<double> tmp(static_cast<size_t>(n) * N), Fmo(static_cast<size_t>(n) * n);
    gbcc::hostla::gemm_tn(n, N, N, h->C.data(), h->F.data(), tmp.data());
    gbcc::hostla::gemm_nn(n, n, N, tmp.data(), h->C.data(), Fmo.data());
    std::vector<double> eo(o), ev(v), Fia(o * v), Fij(o * o), Fab(v * v);
    for (int64_t i = 0; i < o; ++i) eo[i] = Fmo[(fz + i) * n + fz + i];
    for (int64_t a = 0; a < v; ++a) ev[a] = Fmo[(no + a) * n + no + a];
    for (int64_t i = 0; i < o; ++i)
      for (int64_t a = 0; a < v; ++a) Fia[i * v + a] = Fmo[(fz + i) * n + no + a];
    for (int64_t i = 0; i < o; ++i)
      for (int64_t j = 0; j < o; ++j) Fij[i * o + j] = Fmo[(fz + i) * n + fz + j];
    for (int64_t a = 0; a < v; ++a)
      for (int64_t b = 0; b < v; ++b) Fab[a * v + b] = Fmo[(no + a) * n + no + b];
    auto put = [&](const double* dst, const std::vector<double>& src) {
      GBCC_CK(cudaMemcpyAsync(const_cast<double*>(dst), src.data(), src.size() * sizeof(double),
                              cudaMemcpyHostToDevice, st));
    };
    put(in.eps_o, eo);
    put(in.eps_v, ev);
    put(in.Fia, Fia);
    put(in.Fij, Fij);
    put(in.Fab, Fab);
    GBCC_CK(cudaStreamSynchronize(st));
    h->t_tr = now_s() - t0;
    const gbcc_status cs = gbcc_commit_inputs(cc);
    if (cs != GBCC_OK) throw Error(cs, std::string("gbcc_commit_inputs: ") + gbcc_last_error(cc));
    return GBCC_OK;
  });
}

gbcc_status gbcc_scf_destroy(gbcc_scf* h) {
  if (!h) return GBCC_OK;
  cudaSetDevice(h->cfg.device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (void* p : {(void*)h->d_G, (void*)h->d_D, (void*)h->d_J, (void*)h->d_K}) gbcc::dev_free(p);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return GBCC_OK;
}

const char* gbcc_last_scf_error(const gbcc_scf* h) {
  if (!h) return g_scf_create_error.c_str();
  return h->last_error.c_str();
}

int gbcc_testing_eigh(int32_t n, const double* A, double* w, double* V) {
  if (n < 1 || !A || !w || !V) return GBCC_ERR_INVALID_ARG;
  try {
    std::vector<double> a(A, A + static_cast<size_t>(n) * n), ww, vv;
    gbcc::hostla::eigh(n, a, ww, vv);
    std::copy(ww.begin(), ww.end(), w);
    std::copy(vv.begin(), vv.end(), V);
  } catch (const std::exception&) {
    return GBCC_ERR_NUMERIC;
  }
  return GBCC_OK;
}

}  // extern "C"
