// Device integrals of the SCF input producer (ints.cu) and their launchers.
//
// McMurchie-Davidson over contracted Gaussians (s, p, d shells):
//   E^{ab}_{tuv}   Hermite expansion of a primitive pair (host-built, per pair)
//   R_{tuv}        Hermite Coulomb integrals from the Boys function
//   (ab|cd) = 2 pi^{5/2} / (p q sqrt(p+q)) sum E^{ab}_{tuv} (-1)^{tau+nu+phi}
//             E^{cd}_{tau nu phi} R_{t+tau,u+nu,v+phi}(pq/(p+q), P - Q)
// (L. E. McMurchie, E. R. Davidson, J. Comput. Phys. 26, 218 (1978)).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

namespace gbcc {
namespace ints {

constexpr int kLmax = 2;                // s, p, d shells
constexpr int kLpair = 2 * kLmax;       // highest Hermite degree of a pair
constexpr int kLtot = 4 * kLmax;        // highest Hermite degree of a quartet
constexpr int kNhMax = 165;             // (t,u,v) with t+u+v <= 8
constexpr int kNhPair = 35;             // ... <= 4
constexpr int kBoysOrders = kLtot + 7;  // F_0..F_{L+6} per grid point (Taylor terms)
constexpr double kBoysStep = 0.05;      // grid spacing in T
constexpr int kBoysPoints = 801;        // T = 0 .. 40
constexpr double kBoysTmax = 40.0;

__host__ __device__ constexpr int ncart(int l) { return (l + 1) * (l + 2) / 2; }
__host__ __device__ constexpr int nherm(int L) { return (L + 1) * (L + 2) * (L + 3) / 6; }
__host__ __device__ constexpr int pair_class(int l1, int l2) { return l1 * (l1 + 1) / 2 + l2; }  // l1 >= l2
constexpr int kNumPairClasses = pair_class(kLmax, kLmax) + 1;  // 6

// Hermite index of (t,u,v): degree-major, within a degree t descending then u
// descending (host-built tables, the same on both sides)
struct HermTables {
  int8_t t[kNhMax], u[kNhMax], v[kNhMax];
  // recursion of R^n_{tuv} (degree >= 1): first nonzero axis, index of the
  // tuple with that index lowered by one (i1) and by two (i2, or -1), and the
  // coefficient (index - 1) of the second term
  int8_t axis[kNhMax];
  uint8_t i1[kNhMax];
  int16_t i2[kNhMax];
  uint8_t c2[kNhMax];
  // index of h1 + h2 for h1, h2 < kNhPair
  uint8_t sum[kNhPair][kNhPair];
  int16_t tuv[kLtot + 1][kLtot + 1][kLtot + 1];
};
const HermTables& herm_tables();

// F_n(T_k), T_k = k * kBoysStep, n < kBoysOrders (host-built series values)
std::vector<double> boys_table();
// F_0..F_nmax(T) from the series (host; used to build the table)
void boys_series(int nmax, double T, double* F);

// One shell pair, first shell with the larger l.
struct PairInfo {
  int s1, s2;    // shells
  int l1, l2;
  int f1, f2;    // first basis function of each shell
  int nprim;     // primitive pairs
  int prim0;     // first entry in the primitive-pair arrays
  int64_t e0;    // first coefficient in the E data: nprim blocks of [cart pair][nherm(l1+l2)]
};

// exponent sum p and centre P of one primitive pair
struct alignas(32) PrimPair {
  double p, px, py, pz;
};

struct EriArgs {
  const PairInfo* pairs;   // sorted by class
  const PrimPair* prim;    // per primitive pair
  const double* E;         // Hermite coefficients (contraction coefficients folded in)
  const double* boys;      // kBoysPoints x kBoysOrders
  const double* norm;      // per basis function: 1 / sqrt(S_ii) of the unnormalised function
  int nbf;
  int pure;
  int p0, np;              // bra pairs [p0, p0 + np) of one class
  int q0, nq;              // ket pairs of one class
  int same;                // bra and ket class equal: quartets P >= Q only
  int64_t nquart;
  double* G;               // [nbf]^4
};
// (mu nu|la si) of every quartet of shell pairs in class (cP, cQ), cP >= cQ,
// written in all eight permutations
void launch_eri_class(int cP, int cQ, const EriArgs& a, cudaStream_t st);

// Cartesian one-body matrices S, T (kinetic), V (nuclear attraction),
// [ncart_total]^2, unnormalised contracted functions
struct OneBodyArgs {
  int ncart_total;
  const int* cf_shell;     // per Cartesian function: shell
  const int* cf_comp;      // per Cartesian function: (i, j, k) packed as i*16 + j*4 + k
  const int* sh_nprim;
  const int* sh_prim0;
  const double* sh_xyz;    // [nshell][3]
  const double* exps;
  const double* coefs;     // normalised-primitive coefficients x primitive norms
  int natom;
  const double* zn;
  const double* atom_xyz;
  const double* boys;
  double *S, *T, *V;
};
void launch_one_body(const OneBodyArgs& a, cudaStream_t st);

// Fock contributions from the stored (mu nu|la si): J = (mu nu|la si) D_la_si,
// K = (mu la|nu si) D_la_si, deterministic per element.
void launch_coulomb_exchange(int n, const double* G, const double* D, double* J, double* K, cudaStream_t st);

// out[x0][x1][x2][x3] = mo[o + x permuted]: the MO block extraction, with
// mo[p][q][r][s] = (pq|rs) over n orbitals; perm[k] = position in `out` of mo
// index k, off[k] its orbital offset.
void launch_mo_block(int64_t n, const double* mo, const int64_t dims[4], const int perm[4], const int64_t off[4],
                     double* out, cudaStream_t st);

}  // namespace ints
}  // namespace gbcc
