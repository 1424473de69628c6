// kmc_f32.cu -- batched FP32 hop-loop engine for sm_103a: launch validation
// and dispatch (the kernels are in kmc_f32_engine.cuh, instantiated by
// kmc_f32_warp_table.cu, kmc_f32_warp_positions.cu and kmc_f32_block.cu).
//
// A chain is run by a group of threads: a G-lane slice of a warp (G = 4, 8,
// 16, 32; 32/G chains per warp) for small networks, or a whole thread block
// (G = 64 .. 512) for large ones.  Per hop, for every chain:
//
//  pair phase   The allowed transitions are enumerated in the reference's
//               row-major (from, to) order over compact lists: sources are
//               the holes (ascending acceptor index) then the electrodes;
//               a hole's targets are the empty acceptors (ascending) then
//               the electrodes, an electrode's targets the empty acceptors.
//               That is exactly the nonzero part of the reference's dense
//               S x S rate matrix (predicate kmc_dopant_networks.py:137-163,
//               simulation.go:40-55), A(h) = h(N-h) + hP + P(N-h) pairs.
//               The A pairs are split into G contiguous runs, one per
//               thread: balanced runs of ceil(A/G) pairs, or in block groups
//               with long rows, row-aligned runs of whole rows.  Each thread
//               sums its run's Miller-Abrahams rates in FP32:
//                   rate = 2^min(L_ij, L_ij + c B_ij - c (e_j - e_i))
//               L = log2(nu*tc), B = I_0 R / d (acceptor pairs), e = site
//               energies, c = log2(e)/kT: one ex2 per allowed pair
//               (kmc_dopant_networks.py:69-87, simulation.go:58-80).
//               L and B come from a pair table (any tables the caller
//               passes, shared by the chains of one geometry) or, in
//               positions mode, from the sites' coordinates carried in the
//               lists (d from one rsqrt; no table traffic).
//  selection    The per-thread sums become 64-bit integers on a common
//               power-of-two scale and are scanned exactly; the event is the
//               first pair whose cumulative rate reaches u*total
//               (kmc_dopant_networks.py:106-110), u a 64-bit fixed-point
//               uniform with 47 random bits: the exact integer compare picks
//               the thread, then that thread's stored running sums (or its
//               re-evaluated run) are searched relative to its base.
//               The clock advances by Exp(1)/total accumulated in FP64
//               (simulation.go:297-298).
//  hop          O(N) incremental energy update (makeJump,
//               simulation.go:107-130), occupancy bits, electrode counters,
//               optional record (numba or Go convention); every `reanchor`
//               hops the FP32 energies are recomputed from scratch (block
//               groups also carry them compensated in between).
//  site phase   The source/target lists are rebuilt in ascending site order
//               from the occupancy bitmask (popc ranks), carrying each
//               site's scaled energy, ready for the next pair phase.
//
// No tensor cores: nothing here is a contraction.  No spin-waits: every
// loop is bounded by the hop budget or the list sizes.
#include <cstdint>
#include <cuda_runtime.h>

#include "kmc_internal.h"

namespace kmc {

int run_batch(const kmc_batch &b, cudaStream_t st)
{
    if (b.n_chains < 0 || b.n_work < 0 || b.max_sites <= 0 || b.max_sites > kMaxSitesF32)
        return fail(KMC_ERR_INVALID, "engine: bad sizes (n_chains %d, n_work %d, max_sites %d)",
                    b.n_chains, b.n_work, b.max_sites);
    if (b.lanes_per_chain <= 32 && (b.warps_per_block < 1 || b.warps_per_block > 8))
        return fail(KMC_ERR_INVALID, "engine: warps_per_block %d not in 1..8", b.warps_per_block);
    if (b.max_hops_per_launch <= 0)
        return fail(KMC_ERR_INVALID, "engine: max_hops_per_launch must be positive");
    if (b.record < 0 || b.record > 2) return fail(KMC_ERR_INVALID, "engine: bad record mode %d", b.record);
    if (b.record && (!b.occ_time || !b.occ_since || !b.traffic || !b.chain_pair_off))
        return fail(KMC_ERR_INVALID, "engine: record needs occ_time, occ_since, traffic, chain_pair_off");
    if (!b.tab_N || !b.tab_P || !b.chain_tab || !b.chain_kT || !b.chain_site_off ||
        !b.chain_el_off || !b.E_constant || !b.el_energy || !b.occupation ||
        !b.electrode_occupation || !b.time || !b.hops_done || !b.hops_total || !b.stream ||
        !b.status || !b.work)
        return fail(KMC_ERR_INVALID, "engine: a required pointer is NULL");
    if (b.replay && !b.replay_off) return fail(KMC_ERR_INVALID, "engine: replay needs replay_off");
    if (b.lanes_per_chain != 4 && b.lanes_per_chain != 8 && b.lanes_per_chain != 16 && b.lanes_per_chain != 32 &&
        b.lanes_per_chain != 64 && b.lanes_per_chain != 128 && b.lanes_per_chain != 256 && b.lanes_per_chain != 512)
        return fail(KMC_ERR_INVALID, "engine: lanes_per_chain %d not in {4,8,16,32,64,128,256,512}",
                    b.lanes_per_chain);
    if (b.pair_mode == KMC_PAIRS_TABLE) {
        if (!b.tab_off || !b.tab_LB) return fail(KMC_ERR_INVALID, "engine: table mode needs tab_off and tab_LB");
        return b.lanes_per_chain <= 32 ? launch_warp_table(b, st) : launch_block_table(b, st);
    }
    if (b.pair_mode == KMC_PAIRS_POSITIONS) {
        if (!b.tab_pos || !b.tab_pos_off || !b.tab_coef)
            return fail(KMC_ERR_INVALID, "engine: positions mode needs tab_pos, tab_pos_off and tab_coef");
        return b.lanes_per_chain <= 32 ? launch_warp_positions(b, st) : launch_block_positions(b, st);
    }
    return fail(KMC_ERR_INVALID, "engine: bad pair_mode %d", b.pair_mode);
}

int section_clocks(uint64_t *out, int reset)
{
#ifdef KMC_SECTION_CLOCKS
    if (!out) return fail(KMC_ERR_INVALID, "section_clocks: out is NULL");
    for (int k = 0; k < 9; ++k) out[k] = 0;
    int rc;
    if ((rc = section_clocks_warp_table(out, reset)) != KMC_OK) return rc;
    if ((rc = section_clocks_warp_positions(out, reset)) != KMC_OK) return rc;
    return section_clocks_block(out, reset);
#else
    (void)out;
    (void)reset;
    return fail(KMC_ERR_INVALID, "section_clocks: this library was built without -DKMC_SECTION_CLOCKS");
#endif
}

}  // namespace kmc
