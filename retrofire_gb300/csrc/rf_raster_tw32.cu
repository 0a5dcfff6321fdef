// rf_raster_tw32.cu — tile rasteriser kernels for 32-pixel-wide tiles.
#include "rf_raster.cuh"

namespace rfk {
cudaError_t launch_raster_tw32(int kind, bool fast, const JobDev *jobs, uint32_t nj, const DrawDev *draws,
                              const PrimRec *prims, const RasterPrim *rprims, const uint32_t *rows,
                              const uint32_t *tcnt, const uint32_t *toff,
                              const uint32_t *mask, uint32_t ntiles, const uint32_t *items, const uint32_t *nitems,
                          uint32_t *queue,
                              StatsDev *stats, uint32_t warps, int nsm, cudaStream_t s) {
    return launch_raster_for_width<32>(kind, fast, jobs, nj, draws, prims, rprims, rows, tcnt, toff, mask,
                                       ntiles, items, nitems, queue,
                                       stats, warps, nsm, s);
}
}  // namespace rfk
