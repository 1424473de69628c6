// kmc_f32_block.cu -- block-group engine kernels, both pair modes
#include "kmc_f32_engine.cuh"

namespace kmc {

// Block groups (64..512 threads per chain).
int launch_block_table(const kmc_batch &b, cudaStream_t st)
{
    switch (b.lanes_per_chain) {
    case 64: return launch_block<64, TablePairs<false>>(b, st);
    case 128: return launch_block<128, TablePairs<false>>(b, st);
    case 256: return launch_block<256, TablePairs<false>>(b, st);
    case 512: return launch_block<512, TablePairs<false>>(b, st);
    default: return fail(KMC_ERR_INVALID, "engine: %d lanes per chain is not a block group", b.lanes_per_chain);
    }
}

int launch_block_positions(const kmc_batch &b, cudaStream_t st)
{
    switch (b.lanes_per_chain) {
    case 64: return launch_block<64, PairedPositionPairs>(b, st);
    case 128: return launch_block<128, PairedPositionPairs>(b, st);
    case 256: return launch_block<256, PairedPositionPairs>(b, st);
    case 512: return launch_block<512, PairedPositionPairs>(b, st);
    default: return fail(KMC_ERR_INVALID, "engine: %d lanes per chain is not a block group", b.lanes_per_chain);
    }
}

template <int T>
static int preload_size()
{
    int rc;
    if ((rc = preload_block_kernel<T, TablePairs<false>>()) != KMC_OK) return rc;
    if ((rc = preload_block_kernel<T, TablePairs<true>>()) != KMC_OK) return rc;
    return preload_block_kernel<T, PairedPositionPairs>();
}

int preload_block()
{
    int rc;
    if ((rc = preload_size<64>()) != KMC_OK) return rc;
    if ((rc = preload_size<128>()) != KMC_OK) return rc;
    if ((rc = preload_size<256>()) != KMC_OK) return rc;
    return preload_size<512>();
}

int section_clocks_block(uint64_t *out, int reset)
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
