// kmc_f32_warp_table.cu -- warp-slice engine kernels, table mode
#include "kmc_f32_engine.cuh"

namespace kmc {

// Warp slices (4..32 lanes per chain) reading pair tables.
int launch_warp_table(const kmc_batch &b, cudaStream_t st)
{
    switch (b.lanes_per_chain) {
    case 4: return launch_warp<4, TablePairs<false>>(b, st);
    case 8: return launch_warp<8, TablePairs<false>>(b, st);
    case 16: return launch_warp<16, TablePairs<false>>(b, st);
    case 32: return launch_warp<32, TablePairs<false>>(b, st);
    default: return fail(KMC_ERR_INVALID, "engine: %d lanes per chain is not a warp slice", b.lanes_per_chain);
    }
}

template <int G>
static int preload_width()
{
    int rc;
    if ((rc = preload_warp_kernels<G, TablePairs<false>>()) != KMC_OK) return rc;
    if ((rc = preload_warp_kernels<G, TablePairs<true>>()) != KMC_OK) return rc;
    return preload_warp_kernels<G, TablePairs<true, true>>();
}

int preload_warp_table()
{
    int rc;
    if ((rc = preload_width<4>()) != KMC_OK) return rc;
    if ((rc = preload_width<8>()) != KMC_OK) return rc;
    if ((rc = preload_width<16>()) != KMC_OK) return rc;
    return preload_width<32>();
}

int section_clocks_warp_table(uint64_t *out, int reset)
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
