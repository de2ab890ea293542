// Tile-by-tile <-> dense layouts of the boundary's arrays (host side).
//
// MPQC holds every tensor as a TiledArray array over TiledRange1 boundaries
// per dimension (the occupied and virtual tilings of
// src/mpqc/chemistry/qc/lcao/expression/trange1_engine.cpp:10-20, uneven in
// general); an array whose tiles are all local is a sequence of tiles in
// row-major order over the tile grid, each tile row-major over its own
// extents.  The entry points of gbcc.h take dense row-major arrays; these two
// copy between the layouts one contiguous run (a tile row) at a time.
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gbcc.h"

void gbcc_set_thread_error(const std::string& msg);

namespace {

constexpr int kMaxRank = 8;

// validates the boundaries; fills extents and tile counts
bool check_bounds(const char* fn, int32_t rank, const int64_t* const* bounds, const int32_t* nbounds,
                  int64_t* ext, int64_t* ntile) {
  if (rank < 1 || rank > kMaxRank || !bounds || !nbounds) {
    gbcc_set_thread_error(std::string(fn) + ": rank must be 1..8 with boundary arrays");
    return false;
  }
  for (int d = 0; d < rank; ++d) {
    const int64_t* b = bounds[d];
    if (!b || nbounds[d] < 2 || b[0] != 0) {
      gbcc_set_thread_error(std::string(fn) + ": each dimension needs boundaries 0 = b0 < b1 < ... (at least two)");
      return false;
    }
    for (int32_t k = 1; k < nbounds[d]; ++k)
      if (b[k] <= b[k - 1]) {
        gbcc_set_thread_error(std::string(fn) + ": boundaries must increase");
        return false;
      }
    ext[d] = b[nbounds[d] - 1];
    ntile[d] = nbounds[d] - 1;
  }
  return true;
}

// calls run(dense_offset, tiled_offset, length) for every contiguous run
template <typename Run>
void for_each_run(int32_t rank, const int64_t* const* bounds, const int64_t* ext, const int64_t* ntile, Run run) {
  int64_t t[kMaxRank] = {};   // tile multi-index
  int64_t tiled = 0;          // offset of the current tile in the tiled buffer
  for (;;) {
    int64_t lo[kMaxRank], len[kMaxRank], vol = 1;
    for (int d = 0; d < rank; ++d) {
      lo[d] = bounds[d][t[d]];
      len[d] = bounds[d][t[d] + 1] - lo[d];
      vol *= len[d];
    }
    // rows of the tile: every index but the last
    const int64_t rows = vol / len[rank - 1];
    int64_t r[kMaxRank] = {};
    for (int64_t row = 0; row < rows; ++row) {
      int64_t dense = 0;
      for (int d = 0; d < rank - 1; ++d) dense = (dense + lo[d] + r[d]) * ext[d + 1];
      dense += lo[rank - 1];
      run(dense, tiled + row * len[rank - 1], len[rank - 1]);
      for (int d = rank - 2; d >= 0; --d) {
        if (++r[d] < len[d]) break;
        r[d] = 0;
      }
    }
    tiled += vol;
    int d = rank - 1;
    for (; d >= 0; --d) {
      if (++t[d] < ntile[d]) break;
      t[d] = 0;
    }
    if (d < 0) return;
  }
}

}  // namespace

extern "C" {

gbcc_status gbcc_tiles_to_dense(int32_t rank, const int64_t* const* bounds, const int32_t* nbounds,
                                const double* tiles, double* dense) {
  int64_t ext[kMaxRank], ntile[kMaxRank];
  if (!check_bounds("gbcc_tiles_to_dense", rank, bounds, nbounds, ext, ntile)) return GBCC_ERR_INVALID_ARG;
  if (!tiles || !dense) {
    gbcc_set_thread_error("gbcc_tiles_to_dense: NULL array");
    return GBCC_ERR_INVALID_ARG;
  }
  for_each_run(rank, bounds, ext, ntile, [&](int64_t d, int64_t t, int64_t n) {
    std::memcpy(dense + d, tiles + t, static_cast<size_t>(n) * sizeof(double));
  });
  return GBCC_OK;
}

gbcc_status gbcc_dense_to_tiles(int32_t rank, const int64_t* const* bounds, const int32_t* nbounds,
                                const double* dense, double* tiles) {
  int64_t ext[kMaxRank], ntile[kMaxRank];
  if (!check_bounds("gbcc_dense_to_tiles", rank, bounds, nbounds, ext, ntile)) return GBCC_ERR_INVALID_ARG;
  if (!tiles || !dense) {
    gbcc_set_thread_error("gbcc_dense_to_tiles: NULL array");
    return GBCC_ERR_INVALID_ARG;
  }
  for_each_run(rank, bounds, ext, ntile, [&](int64_t d, int64_t t, int64_t n) {
    std::memcpy(tiles + t, dense + d, static_cast<size_t>(n) * sizeof(double));
  });
  return GBCC_OK;
}

}  // extern "C"
