// Fixed-point slice packing of the FP64-grade tensor-core contractions
// (GBCC_PREC_FP64_TC, GatherArgs.fixed): the exponent pass (rowexp[r] = the
// largest biased FP64 exponent of row r of the packed operand) and the digit
// pass, over the same gather expressions and geometries as the BF16 packs.
// A translation unit of its own so the BF16 pack kernels compile as before.
#include "gather.cuh"

namespace gbcc {

namespace {

template <int FIX>
__global__ void __launch_bounds__(256, 4) gather_fixed_rows_kernel(GatherArgs g) {
#define GBCC_ROWS(N, P) gather_rows<N, P, false, FIX>(g)
  GBCC_GATHER_DISPATCH(g, GBCC_ROWS);
#undef GBCC_ROWS
}

template <int FIX>
__global__ void __launch_bounds__(256, 4) gather_fixed4_kernel(GatherArgs g) {
#define GBCC_FIXED4(N, P) split4_rows<N, P, FIX == 1 ? 3 : 4>(g)
  GBCC_GATHER_DISPATCH(g, GBCC_FIXED4);
#undef GBCC_FIXED4
}

template <int FIX>
__global__ void __launch_bounds__(256) gather_fixed_t_kernel(GatherArgs g) {
  __shared__ double tile[32][33];
#define GBCC_TILES(N, P) gather_tiles<N, P, false, FIX>(g, tile)
  GBCC_GATHER_DISPATCH(g, GBCC_TILES);
#undef GBCC_TILES
}

template <int FIX>
void launch_fixed_pass(const GatherArgs& g, cudaStream_t st) {
  const GatherShape sh = gather_shape(g);
  if (sh.kind == GatherShape::kTiles) gather_fixed_t_kernel<FIX><<<sh.grid, sh.block, 0, st>>>(g);
  else if (sh.kind == GatherShape::kFour) gather_fixed4_kernel<FIX><<<sh.grid, sh.block, 0, st>>>(g);
  else gather_fixed_rows_kernel<FIX><<<sh.grid, sh.block, 0, st>>>(g);
}

}  // namespace

void launch_gather_fixed(const GatherArgs& g, cudaStream_t st) {
  if (g.Rpad <= 0 || g.Cpad <= 0 || !g.outs || !g.rowexp) return;
  if (g.fixed == 1) launch_fixed_pass<1>(g, st);
  else launch_fixed_pass<2>(g, st);
}

}  // namespace gbcc
