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
	{10, 51, 2, 4},
	{10, 101, 4, 6},
	{10, 201, 4, 4},
	{15, 51, 4, 4},
	{15, 101, 8, 4},
	{15, 201, 8, 4},
	{20, 51, 8, 6},
	{20, 101, 8, 6},
	{20, 201, 8, 6},
	{25, 51, 8, 8},
	{25, 101, 8, 8},
	{25, 201, 16, 8},
	{30, 51, 8, 8},
	{30, 101, 16, 8},
	{30, 201, 16, 8},
};
#endif
