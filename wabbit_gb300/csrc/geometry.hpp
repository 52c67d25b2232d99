// geometry.hpp -- penalisation masks of a tree drawn from its geometry
// (host side, like the tree bookkeeping: the masks change only with the grid
// and are uploaded after every grid change).
#pragma once
#include <vector>

#include "../../include/wabbit_gb300.h"

namespace wg {

// Interior mask of one block (level, integer coords) in the mask pool's
// layout: 6 components (chi, usx, usy, usz, colour, sponge) of Bs^d points,
// x fastest. Returns whether any word other than the colour is non-zero
// (blocks without such a word run the unmasked stage kernel).
bool geometry_mask_block(const wg_config &cfg, const wg_geometry &geo, int level, const int coords[3],
                         double *out);

// coarseningIndicatorMask_tree's test on one block: 0 where chi has an
// interior point strictly between 1e-12 and 1 - 1e-12 or is not constant
// over the interior, else -1.
int geometry_mask_status(const wg_config &cfg, const wg_geometry &geo, int level, const int coords[3]);

// Checks a geometry against a configuration; returns an error text or "".
const char *geometry_check(const wg_config &cfg, const wg_geometry &geo);

}  // namespace wg
