// kmc_f32_warp_positions.cu -- warp-slice engine kernels, positions mode
#include "kmc_f32_engine.cuh"

namespace kmc {

// Warp slices (4..32 lanes per chain) evaluating distances from coordinates.
int launch_warp_positions(const kmc_batch &b, cudaStream_t st)
{
    switch (b.lanes_per_chain) {
    case 4: return launch_warp<4, PositionPairs>(b, st);
    case 8: return launch_warp<8, PositionPairs>(b, st);
    case 16: return launch_warp<16, PositionPairs>(b, st);
    case 32: return launch_warp<32, PositionPairs>(b, st);
    default: return fail(KMC_ERR_INVALID, "engine: %d lanes per chain is not a warp slice", b.lanes_per_chain);
    }
}

int preload_warp_positions()
{
    int rc;
    if ((rc = preload_warp_kernels<4, PositionPairs>()) != KMC_OK) return rc;
    if ((rc = preload_warp_kernels<8, PositionPairs>()) != KMC_OK) return rc;
    if ((rc = preload_warp_kernels<16, PositionPairs>()) != KMC_OK) return rc;
    return preload_warp_kernels<32, PositionPairs>();
}

int section_clocks_warp_positions(uint64_t *out, int reset)
{
#ifdef KMC_SECTION_CLOCKS
    return section_clocks_read(out, reset);
#else
    (void)out;
    (void)reset;
    return KMC_OK;
#endif
}

}  // namespace kmc
