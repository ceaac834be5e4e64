/*
 * Tile choices per (L, Q) for the mixed-precision path: slices of combos
 * per block of the pipelined translation and gamma pairs per thread of the
 * rotation (0 = the fewest that cover L + 1).  Written by
 * libfmftsaxs_gb300/tune.py from timings on a GB300; a plan takes the entry
 * of the nearest L, then the nearest Q.
 */
#ifndef SXS_TILES_TABLE_H
#define SXS_TILES_TABLE_H
static const struct { int L, Q, tr_slices, rot_gamma; } sxs_tiles_table[] = {
	{20, 101, 8, 0},
};
#endif
