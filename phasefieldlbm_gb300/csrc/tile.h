#pragma once
// Launch geometry shared by the collide kernels and the host code that
// sizes their grids.

// Resident CTAs per SM the collide kernels are compiled for (sets the
// register cap: 65536 / (256 * this)).
#ifndef PFLBM_COLLIDE_MIN_BLOCKS
#define PFLBM_COLLIDE_MIN_BLOCKS 2
#endif

// Column tile of the collide kernels (x fastest; TX a multiple of 32).
#ifndef PFLBM_TILE_X
#define PFLBM_TILE_X 32
#endif
#ifndef PFLBM_TILE_Y
#define PFLBM_TILE_Y 8
#endif

namespace pflbm {
constexpr int kTileX = PFLBM_TILE_X, kTileY = PFLBM_TILE_Y;
static_assert(kTileX % 32 == 0 && kTileX * kTileY <= 1024, "collide tile");
}  // namespace pflbm
