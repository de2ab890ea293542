// A compiled C++ caller of the C ABI (include/gbcc.h, include/gbcc_scf.h), as
// the MPQC shim is: every entry point is called through the headers and
// libgbcc.so alone.  `abi_client cpu` checks the argument and state errors
// every entry point reports (no GPU needed); `abi_client gpu` runs H4 in
// 6-31G end to end: RHF on the GPU, CCSD through the input producer (mixed)
// and through host MO integrals (FP64, gbcc_set_inputs, and the zero-copy
// device inputs), the residual, energy, restarts, (T), a batch and the
// allocation-free energy.  Exit status 0 when every check holds.
#include <cuda_runtime_api.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "gbcc.h"
#include "gbcc_scf.h"

namespace {

int g_failures = 0;

#define CHECK(cond)                                                         \
  do {                                                                      \
    if (!(cond)) {                                                          \
      std::fprintf(stderr, "FAILED %s:%d: %s\n", __FILE__, __LINE__, #cond); \
      ++g_failures;                                                         \
    }                                                                       \
  } while (0)

#define CHECK_OK(call)                                                                      \
  do {                                                                                      \
    const gbcc_status st_ = (call);                                                         \
    if (st_ != GBCC_OK) {                                                                   \
      std::fprintf(stderr, "FAILED %s:%d: %s -> %s\n", __FILE__, __LINE__, #call,            \
                   gbcc_status_string(st_));                                                 \
      ++g_failures;                                                                         \
    }                                                                                       \
  } while (0)

void error_paths(bool gpu) {
  CHECK(gbcc_abi_version() == 6);
  CHECK(std::string(gbcc_status_string(GBCC_ERR_NOT_CONVERGED)) == "not converged");
  gbcc_config c;
  gbcc_config_default(&c);
  CHECK(c.max_iter == 30 && c.n_diis == 8 && c.target_precision == 1e-9);
  CHECK(gbcc_create(nullptr, &c) == GBCC_ERR_INVALID_ARG);
  gbcc_handle* h = nullptr;
  c.o = 0;
  c.v = 4;
  CHECK(gbcc_create(&h, &c) == GBCC_ERR_INVALID_ARG && h == nullptr);
  CHECK(std::strlen(gbcc_last_error(nullptr)) > 0);
  // every handle entry point rejects a NULL handle
  CHECK(gbcc_set_inputs(nullptr, nullptr) == GBCC_ERR_INVALID_ARG);
  CHECK(gbcc_set_df_inputs(nullptr, nullptr) == GBCC_ERR_INVALID_ARG);
  CHECK(gbcc_set_direct_inputs(nullptr, nullptr) == GBCC_ERR_INVALID_ARG);
  CHECK(gbcc_device_inputs(nullptr, nullptr) == GBCC_ERR_INVALID_ARG);
  CHECK(gbcc_commit_inputs(nullptr) == GBCC_ERR_INVALID_ARG);
  CHECK(gbcc_residual(nullptr, nullptr, nullptr, nullptr, nullptr) == GBCC_ERR_INVALID_ARG);
  CHECK(gbcc_residual_ex(nullptr, GBCC_PREC_FP64, nullptr, nullptr, nullptr, nullptr) == GBCC_ERR_INVALID_ARG);
  CHECK(gbcc_energy(nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr) == GBCC_ERR_INVALID_ARG);
  CHECK(gbcc_solve(nullptr, nullptr, nullptr, nullptr, nullptr) == GBCC_ERR_INVALID_ARG);
  CHECK(gbcc_solve_batch(nullptr, 1, nullptr, nullptr, nullptr) == GBCC_ERR_INVALID_ARG);
  CHECK(gbcc_triples(nullptr, GBCC_PREC_FP64, nullptr, nullptr, nullptr) == GBCC_ERR_INVALID_ARG);
  CHECK(gbcc_set_amplitudes(nullptr, nullptr, nullptr) == GBCC_ERR_INVALID_ARG);
  CHECK(gbcc_save_amplitudes(nullptr, "x") == GBCC_ERR_INVALID_ARG);
  CHECK(gbcc_load_amplitudes(nullptr, "x", nullptr) == GBCC_ERR_INVALID_ARG);
  int32_t sl[3];
  double rc[3];
  CHECK(gbcc_slice_policy(nullptr, sl, rc) == GBCC_ERR_INVALID_ARG);
  CHECK(gbcc_calibrate_slices(nullptr, nullptr, nullptr) == GBCC_ERR_INVALID_ARG);
  CHECK(gbcc_destroy(nullptr) == GBCC_OK);
  double out[2];
  CHECK(gbcc_energy_noalloc(0, 8, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, out, nullptr) ==
        GBCC_ERR_INVALID_ARG);
  CHECK(gbcc_energy_noalloc(4, 513, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, out, nullptr) ==
        GBCC_ERR_INVALID_ARG);
  CHECK(gbcc_autotune_load(nullptr) == GBCC_ERR_INVALID_ARG);
  CHECK(gbcc_autotune_save(nullptr) == GBCC_ERR_INVALID_ARG);
  CHECK(gbcc_autotune_clear() == GBCC_OK);
  // tile-layout adapters (host only): a 5 x 4 array in tiles of rows {2, 3} x columns {1, 3}
  {
    const int64_t b0[] = {0, 2, 5}, b1[] = {0, 1, 4};
    const int64_t* bounds[] = {b0, b1};
    const int32_t nb[] = {3, 3};
    double dense[20], back[20], tiles[20];
    for (int k = 0; k < 20; ++k) dense[k] = k;
    CHECK(gbcc_dense_to_tiles(2, bounds, nb, dense, tiles) == GBCC_OK);
    // first tile: rows 0-1, column 0; second: rows 0-1, columns 1-3
    CHECK(tiles[0] == 0 && tiles[1] == 4 && tiles[2] == 1 && tiles[3] == 2 && tiles[4] == 3 && tiles[5] == 5);
    CHECK(gbcc_tiles_to_dense(2, bounds, nb, tiles, back) == GBCC_OK);
    CHECK(std::memcmp(dense, back, sizeof(dense)) == 0);
    CHECK(gbcc_tiles_to_dense(0, bounds, nb, tiles, back) == GBCC_ERR_INVALID_ARG);
    CHECK(gbcc_dense_to_tiles(2, bounds, nb, nullptr, tiles) == GBCC_ERR_INVALID_ARG);
  }
  // input producer
  gbcc_scf_config sc;
  gbcc_scf_config_default(&sc);
  CHECK(sc.max_iter == 30);
  gbcc_scf* scf = nullptr;
  CHECK(gbcc_scf_create(&scf, nullptr, nullptr, &sc) == GBCC_ERR_INVALID_ARG && scf == nullptr);
  CHECK(std::strlen(gbcc_last_scf_error(nullptr)) > 0);
  CHECK(gbcc_scf_run(nullptr, nullptr) == GBCC_ERR_INVALID_ARG);
  CHECK(gbcc_scf_ao(nullptr, nullptr, nullptr, nullptr) == GBCC_ERR_INVALID_ARG);
  CHECK(gbcc_scf_orbitals(nullptr, nullptr, nullptr) == GBCC_ERR_INVALID_ARG);
  CHECK(gbcc_scf_ccsd_inputs(nullptr, 0, nullptr) == GBCC_ERR_INVALID_ARG);
  CHECK(gbcc_scf_destroy(nullptr) == GBCC_OK);
  if (!gpu) {
    // no device: creation fails cleanly and returns no handle
    gbcc_config_default(&c);
    c.o = 2;
    c.v = 3;
    CHECK(gbcc_create(&h, &c) == GBCC_ERR_CUDA && h == nullptr);
  }
}

// H4: two H2 (1.4 bohr) 3 bohr apart, 6-31G (published Ditchfield-Hehre-Pople
// exponents and contraction coefficients)
struct H4 {
  double charge[4] = {1, 1, 1, 1};
  double xyz[12] = {0, 0, 0, 0, 0, 1.4, 3.0, 0, 0, 3.0, 0, 1.4};
  int32_t atom[8] = {0, 0, 1, 1, 2, 2, 3, 3};
  int32_t l[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  int32_t nprim[8] = {3, 1, 3, 1, 3, 1, 3, 1};
  std::vector<double> exps, coefs;
  H4() {
    for (int a = 0; a < 4; ++a) {
      exps.insert(exps.end(), {18.7311370, 2.8253937, 0.6401217, 0.1612778});
      coefs.insert(coefs.end(), {0.03349460, 0.23472695, 0.81375733, 1.0});
    }
  }
};

double solve(gbcc_handle* h, std::vector<double>* t1, std::vector<double>* t2, gbcc_report* rep) {
  double e = 0.0;
  CHECK_OK(gbcc_solve(h, t1 ? t1->data() : nullptr, t2 ? t2->data() : nullptr, &e, rep));
  return e;
}

void end_to_end() {
  H4 m;
  gbcc_molecule mol{4, m.charge, m.xyz, 0};
  gbcc_basis bas{8, m.atom, m.l, m.nprim, m.exps.data(), m.coefs.data(), 0};
  gbcc_scf_config sc;
  gbcc_scf_config_default(&sc);
  gbcc_scf* scf = nullptr;
  CHECK_OK(gbcc_scf_create(&scf, &mol, &bas, &sc));
  gbcc_scf_report sr{};
  CHECK_OK(gbcc_scf_run(scf, &sr));
  CHECK(sr.converged && sr.nbf == 8 && sr.nocc == 2 && sr.energy < -1.0);
  const int n = sr.nbf, o = sr.nocc, v = n - o;
  std::vector<double> S(n * n), H(n * n), G(static_cast<size_t>(n) * n * n * n), C(n * n), eps(n);
  CHECK_OK(gbcc_scf_ao(scf, S.data(), H.data(), G.data()));
  CHECK_OK(gbcc_scf_orbitals(scf, C.data(), eps.data()));

  // (1) mixed precision through the input producer
  gbcc_config c;
  gbcc_config_default(&c);
  c.o = o;
  c.v = v;
  c.precision = GBCC_PREC_MIXED;
  c.target_precision = 1e-10;
  gbcc_handle* hm = nullptr;
  CHECK_OK(gbcc_create(&hm, &c));
  CHECK_OK(gbcc_scf_ccsd_inputs(scf, 0, hm));
  gbcc_report rm{};
  const double em = solve(hm, nullptr, nullptr, &rm);
  CHECK(rm.converged && em < 0.0);

  // (2) FP64 from host MO integrals: (pq|rs) = sum C C C C (mu nu|la si)
  std::vector<double> mo(static_cast<size_t>(n) * n * n * n, 0.0), tmp(mo.size(), 0.0);
  auto I4 = [n](int p, int q, int r, int s) { return ((static_cast<size_t>(p) * n + q) * n + r) * n + s; };
  for (int p = 0; p < n; ++p)  // first index
    for (int b = 0; b < n; ++b)
      for (int c2 = 0; c2 < n; ++c2)
        for (int d = 0; d < n; ++d) {
          double s = 0;
          for (int a = 0; a < n; ++a) s += C[a * n + p] * G[I4(a, b, c2, d)];
          tmp[I4(p, b, c2, d)] = s;
        }
  for (int p = 0; p < n; ++p)
    for (int q = 0; q < n; ++q)
      for (int c2 = 0; c2 < n; ++c2)
        for (int d = 0; d < n; ++d) {
          double s = 0;
          for (int b = 0; b < n; ++b) s += C[b * n + q] * tmp[I4(p, b, c2, d)];
          mo[I4(p, q, c2, d)] = s;
        }
  for (int p = 0; p < n; ++p)
    for (int q = 0; q < n; ++q)
      for (int r = 0; r < n; ++r)
        for (int d = 0; d < n; ++d) {
          double s = 0;
          for (int c2 = 0; c2 < n; ++c2) s += C[c2 * n + r] * mo[I4(p, q, c2, d)];
          tmp[I4(p, q, r, d)] = s;
        }
  for (int p = 0; p < n; ++p)
    for (int q = 0; q < n; ++q)
      for (int r = 0; r < n; ++r)
        for (int s2 = 0; s2 < n; ++s2) {
          double s = 0;
          for (int d = 0; d < n; ++d) s += C[d * n + s2] * tmp[I4(p, q, r, d)];
          mo[I4(p, q, r, s2)] = s;
        }
  auto chem = [&](int p, int q, int r, int s) { return mo[I4(p, q, r, s)]; };  // (pq|rs)
  // <pq|rs> = (pr|qs), MPQC annotation order, virtual indices offset by o
  std::vector<double> eo(eps.begin(), eps.begin() + o), ev(eps.begin() + o, eps.end());
  std::vector<double> Fia(o * v, 0.0), Fij(o * o, 0.0), Fab(v * v, 0.0);
  for (int i = 0; i < o; ++i) Fij[i * o + i] = eo[i];
  for (int a = 0; a < v; ++a) Fab[a * v + a] = ev[a];
  std::vector<double> Gijab(o * o * v * v), Gijkl(o * o * o * o), Giajb(o * v * o * v), Gijka(o * o * o * v),
      Giabc(o * v * v * v), Gabcd(v * v * v * v);
  for (int i = 0; i < o; ++i)
    for (int j = 0; j < o; ++j) {
      for (int a = 0; a < v; ++a)
        for (int b = 0; b < v; ++b) Gijab[((i * o + j) * v + a) * v + b] = chem(i, o + a, j, o + b);
      for (int k = 0; k < o; ++k) {
        for (int l2 = 0; l2 < o; ++l2) Gijkl[((i * o + j) * o + k) * o + l2] = chem(i, k, j, l2);
        for (int a = 0; a < v; ++a) Gijka[((i * o + j) * o + k) * v + a] = chem(i, k, j, o + a);
      }
    }
  for (int i = 0; i < o; ++i)
    for (int a = 0; a < v; ++a) {
      for (int j = 0; j < o; ++j)
        for (int b = 0; b < v; ++b) Giajb[((i * v + a) * o + j) * v + b] = chem(i, j, o + a, o + b);
      for (int b = 0; b < v; ++b)
        for (int c2 = 0; c2 < v; ++c2) Giabc[((i * v + a) * v + b) * v + c2] = chem(i, o + b, o + a, o + c2);
    }
  for (int a = 0; a < v; ++a)
    for (int b = 0; b < v; ++b)
      for (int c2 = 0; c2 < v; ++c2)
        for (int d = 0; d < v; ++d) Gabcd[((a * v + b) * v + c2) * v + d] = chem(o + a, o + c2, o + b, o + d);
  gbcc_inputs in{eo.data(), ev.data(), Fia.data(), Fij.data(), Fab.data(), Gijab.data(),
                 Gijkl.data(), Giajb.data(), Gijka.data(), Giabc.data(), Gabcd.data()};
  c.precision = GBCC_PREC_FP64;
  gbcc_handle* hf = nullptr;
  CHECK_OK(gbcc_create(&hf, &c));
  CHECK(gbcc_residual(hf, nullptr, nullptr, nullptr, nullptr) != GBCC_OK);  // no inputs yet
  CHECK_OK(gbcc_set_inputs(hf, &in));
  std::vector<double> t1(v * o), t2(v * v * o * o);
  gbcc_report rf{};
  const double ef = solve(hf, &t1, &t2, &rf);
  CHECK(rf.converged && rf.mixed_iters == 0);
  CHECK(std::fabs(ef - em) < 1e-8);

  // restarts: checkpoint file and seeded amplitudes
  const std::string path = std::string(std::getenv("GBCC_CLIENT_TMP") ? std::getenv("GBCC_CLIENT_TMP") : ".") +
                           "/abi_client_amplitudes.bin";
  CHECK_OK(gbcc_save_amplitudes(hf, path.c_str()));
  double eload = 0;
  CHECK_OK(gbcc_load_amplitudes(hf, path.c_str(), &eload));
  CHECK(eload == ef);
  CHECK_OK(gbcc_set_amplitudes(hf, t1.data(), t2.data()));
  gbcc_report rr{};
  const double er = solve(hf, nullptr, nullptr, &rr);
  CHECK(rr.converged && rr.iters <= 3 && std::fabs(er - ef) < 1e-9);
  std::remove(path.c_str());

  // (T) from the last solve's amplitudes
  double et = 0;
  CHECK_OK(gbcc_triples(hf, GBCC_PREC_FP64, nullptr, nullptr, &et));
  CHECK(et < 0.0 && et > -0.01);

  // residual and energy at the converged amplitudes
  std::vector<double> r1(v * o), r2(v * v * o * o);
  CHECK_OK(gbcc_residual(hf, t1.data(), t2.data(), r1.data(), r2.data()));
  double e = 0, err = 1;
  CHECK_OK(gbcc_energy(hf, t1.data(), t2.data(), r1.data(), r2.data(), &e, &err));
  CHECK(std::fabs(e - ef) < 1e-9 && err < 1e-8);
  CHECK_OK(gbcc_residual_ex(hm, GBCC_PREC_FP64, t1.data(), t2.data(), r1.data(), r2.data()));
  CHECK(gbcc_residual_ex(hm, GBCC_PREC_FP64_TC, t1.data(), t2.data(), r1.data(), r2.data()) == GBCC_ERR_STATE);
  CHECK(std::strlen(gbcc_last_error(hm)) > 0);
  int32_t sl[3];
  double rc[3];
  CHECK_OK(gbcc_slice_policy(hm, sl, rc));
  CHECK(sl[0] >= 1 && sl[0] <= 3);
  CHECK_OK(gbcc_calibrate_slices(hm, t1.data(), t2.data()));

  // zero-copy inputs: the handle's own device arrays, filled here
  gbcc_handle* hz = nullptr;
  CHECK_OK(gbcc_create(&hz, &c));
  gbcc_inputs dev{};
  CHECK_OK(gbcc_device_inputs(hz, &dev));
  auto put = [](const double* d, const std::vector<double>& h) {
    CHECK(cudaMemcpy(const_cast<double*>(d), h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice) ==
          cudaSuccess);
  };
  put(dev.eps_o, eo);
  put(dev.eps_v, ev);
  put(dev.Fia, Fia);
  put(dev.Fij, Fij);
  put(dev.Fab, Fab);
  put(dev.Gijab, Gijab);
  put(dev.Gijkl, Gijkl);
  put(dev.Giajb, Giajb);
  put(dev.Gijka, Gijka);
  put(dev.Giabc, Giabc);
  put(dev.Gabcd, Gabcd);
  CHECK_OK(gbcc_commit_inputs(hz));
  const double ez = solve(hz, nullptr, nullptr, nullptr);
  CHECK(std::fabs(ez - ef) < 1e-10);

  // batch of two handles
  gbcc_handle* both[2] = {hm, hz};
  double eb[2] = {0, 0};
  gbcc_report rb[2];
  gbcc_status sb[2];
  CHECK_OK(gbcc_solve_batch(both, 2, eb, rb, sb));
  CHECK(sb[0] == GBCC_OK && sb[1] == GBCC_OK && std::fabs(eb[1] - ez) < 1e-12 && std::fabs(eb[0] - em) < 1e-8);

  // allocation-free energy on device copies of the converged state
  {
    std::vector<double> f_ai(v * o, 0.0), g_abij(v * v * o * o), tau(t2);
    for (int a = 0; a < v; ++a)
      for (int b = 0; b < v; ++b)
        for (int i = 0; i < o; ++i)
          for (int j = 0; j < o; ++j) {
            g_abij[((a * v + b) * o + i) * o + j] = Gijab[((i * o + j) * v + a) * v + b];
            tau[((a * v + b) * o + i) * o + j] += t1[a * o + i] * t1[b * o + j];
          }
    CHECK_OK(gbcc_residual(hf, t1.data(), t2.data(), r1.data(), r2.data()));
    const std::vector<const std::vector<double>*> host = {&f_ai, &g_abij, &t1, &tau, &r1, &r2};
    std::vector<double*> d(7, nullptr);
    for (size_t k = 0; k < host.size(); ++k) {
      CHECK(cudaMalloc(reinterpret_cast<void**>(&d[k]), host[k]->size() * sizeof(double)) == cudaSuccess);
      CHECK(cudaMemcpy(d[k], host[k]->data(), host[k]->size() * sizeof(double), cudaMemcpyHostToDevice) ==
            cudaSuccess);
    }
    CHECK(cudaMalloc(reinterpret_cast<void**>(&d[6]), 2 * sizeof(double)) == cudaSuccess);
    CHECK_OK(gbcc_energy_noalloc(o, v, d[0], d[1], d[2], d[3], d[4], d[5], d[6], nullptr));
    double eo2[2];
    CHECK(cudaMemcpy(eo2, d[6], sizeof(eo2), cudaMemcpyDeviceToHost) == cudaSuccess);
    double e2 = 0, err2 = 0;
    CHECK_OK(gbcc_energy(hf, t1.data(), t2.data(), r1.data(), r2.data(), &e2, &err2));
    CHECK(std::fabs(eo2[0] - e2) < 1e-12 && std::fabs(eo2[1] - err2) < 1e-15);
    // host memory is rejected
    CHECK(gbcc_energy_noalloc(o, v, f_ai.data(), d[1], d[2], d[3], d[4], d[5], d[6], nullptr) ==
          GBCC_ERR_INVALID_ARG);
    for (double* p : d) cudaFree(p);
  }

  // the other input forms reject missing arrays
  gbcc_df_inputs dfi{};
  CHECK(gbcc_set_df_inputs(hf, &dfi) == GBCC_ERR_INVALID_ARG);
  gbcc_direct_inputs dri{};
  CHECK(gbcc_set_direct_inputs(hf, &dri) == GBCC_ERR_INVALID_ARG);

  // autotune table of the mixed handle's contractions
  const std::string tpath = path + ".tune";
  CHECK_OK(gbcc_autotune_save(tpath.c_str()));
  CHECK_OK(gbcc_autotune_clear());
  CHECK_OK(gbcc_autotune_load(tpath.c_str()));
  std::remove(tpath.c_str());

  CHECK_OK(gbcc_destroy(hz));
  CHECK_OK(gbcc_destroy(hf));
  CHECK_OK(gbcc_destroy(hm));
  CHECK_OK(gbcc_scf_destroy(scf));
  std::printf("H4/6-31G: E_RHF %.10f E_CCSD(mixed) %.10f E_CCSD(FP64) %.10f E(T) %.10f\n", sr.energy, em, ef, et);
}

}  // namespace

int main(int argc, char** argv) {
  const bool gpu = argc > 1 && std::strcmp(argv[1], "gpu") == 0;
  error_paths(gpu);
  if (gpu) end_to_end();
  if (g_failures) {
    std::fprintf(stderr, "%d check(s) failed\n", g_failures);
    return 1;
  }
  std::printf("abi_client %s: all checks passed\n", gpu ? "gpu" : "cpu");
  return 0;
}
