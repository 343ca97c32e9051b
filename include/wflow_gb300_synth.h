/*
 * wflow_gb300_synth.h -- seeded synthetic catchment generator (host library
 * libwflow_synth.so), the stand-in for Wflow's staticmaps netCDF in benchmarks and tests.
 *
 * It has no counterpart in the reference (Wflow.jl reads real maps); it produces the D8
 * network the reference builds with flowgraph (Wflow/src/routing/utils.jl:6-33) from a
 * PCRaster LDD, with flow length/width as in Wflow/src/utils.jl:418-449.
 */
#ifndef WFLOW_GB300_SYNTH_H
#define WFLOW_GB300_SYNTH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Fractal DEM (diamond-square with amplitude ratio `scale_ratio` = 2^-H per level) plus a plane
 * dipping to the outlet corner with `tilt` times the fractal relief, rescaled to [0, zmax],
 * priority-flood pit filling with an epsilon gradient towards the single outlet at
 * cell (0, 0), D8 steepest descent (PCRaster codes 1-9), downstream index (-1 at the outlet),
 * slope (>= min_slope), upstream cell counts (including the cell). Cell index = y * nx + x.
 * Returns 0 on success. */
int32_t wf_synth_dem_d8(int32_t nx, int32_t ny, uint64_t seed, double scale_ratio, double zmax,
                        double cell_size, double min_slope, double tilt, double* dem, uint8_t* ldd,
                        int32_t* downstream, double* slope, int64_t* upstream_cells,
                        double* flow_length, double* flow_width);

#ifdef __cplusplus
}
#endif

#endif
