/* Seeded synthetic inputs for the reconstruction / labelling path (host-only helpers).
 *
 * These have no counterpart in the reference: its tests read pathology tiles from a data
 * directory that it does not ship (test/TestUtils.h:9-17).  The generator produces tiles
 * of the same shape and value ranges (bright noisy background, dark elliptical nuclei);
 * the full definition is at the top of csrc/synth.cpp.  All functions return 0 on success
 * and -1 on a bad argument.
 */
#ifndef NSGB_SYNTH_H_
#define NSGB_SYNTH_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* mask: H x W u8 (row pitch in elements) with n_ellipses dark ellipses; marker (optional,
 * same pitch) = max(mask - 10, 0). */
int nsgb_synth_tile_u8(uint8_t* mask, uint8_t* marker, int64_t H, int64_t W, int64_t pitch,
                       int64_t n_ellipses, uint64_t seed);
/* u16 tile from a u8 tile: value * 257, marker = max(value*257 - 2570, 0). */
int nsgb_synth_scale_u16(const uint8_t* src, uint16_t* mask, uint16_t* marker, int64_t n);
/* i32 tile from a u8 tile: value * 1000, marker = max(value*1000 - 10000, 0). */
int nsgb_synth_scale_i32(const uint8_t* src, int32_t* mask, int32_t* marker, int64_t n);
/* f32: mask uniform in [0,1) on a 2^-24 grid; marker = mask * u, u uniform in [0.5, 1). */
int nsgb_synth_float(float* mask, float* marker, int64_t n, uint64_t seed);
/* Tile sizes for the uneven batch: heights/widths uniform in [lo, hi]. */
int nsgb_synth_tile_sizes(int32_t* heights, int32_t* widths, int64_t n_tiles, int32_t lo,
                          int32_t hi, uint64_t seed);

#ifdef __cplusplus
}
#endif

#endif /* NSGB_SYNTH_H_ */
