// kmc_f32.cu -- batched FP32 hop-loop engine for sm_103a.
//
// One chain per group of G lanes (G = 4, 8, 16 or 32; 32/G chains per warp).
// Per hop, for every chain:
//
//  pair phase   The allowed transitions are enumerated in the reference's
//               row-major (from, to) order over compact lists: sources are
//               the holes (ascending acceptor index) then the electrodes;
//               a hole's targets are the empty acceptors (ascending) then
//               the electrodes, an electrode's targets the empty acceptors.
//               That is exactly the nonzero part of the reference's dense
//               S x S rate matrix (predicate kmc_dopant_networks.py:137-163,
//               simulation.go:40-55), A(h) = h(N-h) + hP + P(N-h) pairs.
//               Lane g owns the contiguous run [g*M, g*M+M) of the A pairs
//               and sums its Miller-Abrahams rates in FP32:
//                   rate = 2^(L_ij - c*max(0, e_j - e_i - B_ij))
//               with L = log2(nu*tc), B = I_0 R / d (acceptor pairs),
//               e = energies, c = log2(e)/kT: one ex2 per allowed pair
//               (kmc_dopant_networks.py:69-87, simulation.go:58-80).
//  selection    The G lane sums are scanned in FP64; the clock advances by
//               Exp(1)/total accumulated in FP64 (simulation.go:297-298);
//               the event is the first pair whose cumulative rate reaches
//               u*total (kmc_dopant_networks.py:106-110): the FP64 compare
//               picks the lane, then the lane's run is re-evaluated by the
//               group and scanned relative to that lane's FP64 base.
//  hop          O(N) incremental energy update (makeJump,
//               simulation.go:107-130), occupancy bits, electrode counters,
//               optional record (numba or Go convention); every `reanchor`
//               hops the FP32 energies are recomputed from scratch so the
//               rounding of the incremental updates cannot drift.
//  site phase   The source/target lists are rebuilt in ascending site order
//               from the occupancy bitmask (popc ranks), carrying each
//               site's scaled energy, ready for the next pair phase.
//
// Pair tables are read through the read-only data path (L1/L2 resident for
// shared geometries).  No tensor cores: nothing here is a contraction.
#include <cstdint>
#include <cstdio>
#include <cuda_runtime.h>

#include "kmc_common.cuh"
#include "kmc_internal.h"

namespace kmc {
namespace {

constexpr float kLog2e = 1.4426950408889634f;
constexpr int kMaxElectrodes = 64;

__device__ __forceinline__ float ex2_approx(float x)
{
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// k -> (row, col) within the pair enumeration.  Float-reciprocal quotient
// with one correction step; exact for k < 2^22 (the engine limits S so that
// A(h) stays below that).
__device__ __forceinline__ void decode_pair(int k, int h, int A1, int T1, int T2, float inv1,
                                            float inv2, int &row, int &col)
{
    if (k < A1) {
        int q = __float2int_rz(__int2float_rn(k) * inv1);
        int r = k - q * T1;
        if (r < 0) { --q; r += T1; } else if (r >= T1) { ++q; r -= T1; }
        row = q;
        col = r;
    } else {
        const int kk = k - A1;
        int q = __float2int_rz(__int2float_rn(kk) * inv2);
        int r = kk - q * T2;
        if (r < 0) { --q; r += T2; } else if (r >= T2) { ++q; r -= T2; }
        row = h + q;
        col = r;
    }
}

struct ChainSmem {
    int2 *src;        // [S+1] {site, scaled energy bits}
    int2 *tgt;        // [S+1]
    float *E;         // [S]   site energies (acceptors)
    uint32_t *occw;   // [W]   occupancy bits
    int *eo;          // [kMaxElectrodes] electrode counters of this launch
};

__host__ __device__ __forceinline__ int chain_smem_words(int S)
{
    const int W = (S + 31) / 32;
    int words = 2 * (S + 1) + 2 * (S + 1) + S + W + kMaxElectrodes;
    return (words + 3) & ~3;
}

__device__ __forceinline__ ChainSmem carve(uint32_t *base, int S)
{
    ChainSmem c;
    c.src = reinterpret_cast<int2 *>(base);
    c.tgt = c.src + (S + 1);
    c.E = reinterpret_cast<float *>(c.tgt + (S + 1));
    c.occw = reinterpret_cast<uint32_t *>(c.E + S);
    c.eo = reinterpret_cast<int *>(c.occw + (S + 31) / 32);
    return c;
}

// Rate of pair (source record s, target record t): one ex2.
__device__ __forceinline__ float pair_rate(const float2 *__restrict__ tab, int S, int2 s, int2 t,
                                           float cs)
{
    const float2 lb = __ldg(&tab[s.x * S + t.x]);
    float x = __int_as_float(t.y) - __int_as_float(s.y);
    x = fmaf(-cs, lb.y, x);
    x = fmaxf(x, 0.0f);
    return ex2_approx(lb.x - x);
}

template <int G>
__global__ void __launch_bounds__(256) f32_engine_kernel(const kmc_batch B)
{
    constexpr int CPW = 32 / G;
    extern __shared__ __align__(16) uint32_t smem[];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int sub = lane / G;
    const int g = lane % G;
    const unsigned gmask = (G == 32 ? 0xffffffffu : ((1u << G) - 1u)) << (sub * G);
    const int Smax = B.max_sites;
    const int item = blockIdx.x * B.warps_per_block + warp;
    if (item >= B.n_work) return;
    const int c = B.work[item * CPW + sub];
    if (c < 0 || c >= B.n_chains) return;   // whole group leaves together

    ChainSmem sm = carve(smem + (warp * CPW + sub) * chain_smem_words(Smax), Smax);

    const int t_id = B.chain_tab[c];
    const int N = B.tab_N[t_id];
    const int P = B.tab_P[t_id];
    const int S = N + P;
    const float2 *tab = reinterpret_cast<const float2 *>(B.tab_LB + B.tab_off[t_id]);
    const int64_t so = B.chain_site_off[c];
    const int64_t eoff = B.chain_el_off[c];
    const float *Ec = B.E_constant + so;
    const float *Vel = B.el_energy + eoff;
    uint8_t *occ_g = B.occupation + so;
    const float kT = B.chain_kT[c];
    const float cs = kLog2e / kT;
    const int64_t hops_done0 = B.hops_done[c];
    int64_t todo = B.hops_total[c] - hops_done0;
    if (todo > B.max_hops_per_launch) todo = B.max_hops_per_launch;
    const uint64_t stream = B.stream[c];
    const uint32_t k0 = static_cast<uint32_t>(B.seed), k1 = static_cast<uint32_t>(B.seed >> 32);
    const int record = B.record;
    const int reanchor = B.reanchor > 0 ? B.reanchor : 1024;
    const int W = (N + 31) / 32;
    if (P > kMaxElectrodes || S > Smax || N < 0) {
        if (g == 0) B.status[c] = KMC_ERR_INVALID;
        return;
    }

    // ---- load state ----
    for (int w = g; w < W; w += G) {
        uint32_t bits = 0;
        for (int b = 0; b < 32; ++b) {
            const int j = w * 32 + b;
            if (j < N && occ_g[j]) bits |= 1u << b;
        }
        sm.occw[w] = bits;
    }
    for (int e = g; e < P; e += G) sm.eo[e] = 0;
    __syncwarp(gmask);
    int h = 0;
    for (int w = 0; w < W; ++w) h += __popc(sm.occw[w]);

    double t = B.time[c];
    int64_t hop = hops_done0;
    const int64_t hop_end = hops_done0 + (todo > 0 ? todo : 0);
    int status = KMC_OK;
    unsigned long long pairs = 0;
    const double *replay = B.replay ? B.replay + B.replay_off[c] : nullptr;
    double *occ_time = record ? B.occ_time + so : nullptr;
    double *occ_since = record ? B.occ_since + so : nullptr;
    int32_t *traffic = record ? B.traffic + B.chain_pair_off[c] : nullptr;
    if (record) {
        for (int j = g; j < N; j += G) occ_since[j] = t;
    }

    u32x4 rnd{0, 0, 0, 0};
    int64_t rbase = INT64_MIN / 2;
    bool need_anchor = true;

    while (hop < hop_end) {
        if (B.cancel && (hop & 1023) == 0) {
            // one read per group, broadcast, so the group leaves together
            const int stop = __shfl_sync(gmask, g == 0 ? *B.cancel : 0, 0, G);
            if (stop) { status = KMC_ERR_CANCELLED; break; }
        }
        // ---- (re)anchor energies: E_j = Ec_j - sum_{k empty} B_jk ----
        if (need_anchor || (hop % reanchor) == 0) {
            for (int j = g; j < N; j += G) {
                float acc = 0.0f;
                const float2 *row = tab + j * S;
                for (int k = 0; k < N; ++k)
                    if (!((sm.occw[k >> 5] >> (k & 31)) & 1u)) acc += __ldg(&row[k]).y;
                sm.E[j] = Ec[j] - acc;
            }
            need_anchor = false;
            __syncwarp(gmask);
        }
        // ---- site phase: rebuild ordered source / target lists ----
        {
            const int z = N - h;
            int wcur = 0, cum = 0;
            for (int j = g; j < N; j += G) {
                const int w = j >> 5;
                while (wcur < w) { cum += __popc(sm.occw[wcur]); ++wcur; }
                const uint32_t word = sm.occw[w];
                const int below = cum + __popc(word & ((1u << (j & 31)) - 1u));
                const int2 rec = make_int2(j, __float_as_int(cs * sm.E[j]));
                if ((word >> (j & 31)) & 1u) sm.src[below] = rec;
                else sm.tgt[j - below] = rec;
            }
            for (int e = g; e < P; e += G) {
                const int2 rec = make_int2(N + e, __float_as_int(cs * Vel[e]));
                sm.src[h + e] = rec;
                sm.tgt[z + e] = rec;
            }
            __syncwarp(gmask);
        }
        // ---- pair phase ----
        const int z = N - h;
        const int T1 = z + P, T2 = z;
        const int A1 = h * T1;
        const int A = A1 + P * T2;
        if (A <= 0) { status = KMC_ERR_NONFINITE; break; }
        const float inv1 = T1 > 0 ? 1.0f / T1 : 0.0f;
        const float inv2 = T2 > 0 ? 1.0f / T2 : 0.0f;
        const int M = (A + G - 1) / G;
        float lsum = 0.0f;
        {
            const int kb = g * M;
            const int ke = min(kb + M, A);
            if (kb < ke) {
                int row, col;
                decode_pair(kb, h, A1, T1, T2, inv1, inv2, row, col);
                int Tcur = row < h ? T1 : T2;
                int2 sr = sm.src[row];
                for (int k = kb; k < ke; ++k) {
                    lsum += pair_rate(tab, S, sr, sm.tgt[col], cs);
                    if (++col == Tcur) {
                        col = 0;
                        ++row;
                        Tcur = row < h ? T1 : T2;
                        sr = sm.src[row];
                    }
                }
            }
        }
        pairs += static_cast<unsigned long long>(A);
        // ---- uniforms for this hop ----
        double u_ev;
        float e1;
        if (replay) {
            const double u1 = replay[2 * hop], u2 = replay[2 * hop + 1];
            e1 = -log1pf(-static_cast<float>(u1));
            u_ev = u2;
        } else {
            if (hop - rbase >= G) {
                rbase = hop;
                const uint64_t ctr = static_cast<uint64_t>(hop + g);
                rnd = philox4x32_10(u32x4{static_cast<uint32_t>(ctr), static_cast<uint32_t>(ctr >> 32),
                                          static_cast<uint32_t>(stream),
                                          static_cast<uint32_t>(stream >> 32)},
                                    k0, k1);
            }
            const int ri = static_cast<int>(hop - rbase);
            const uint32_t w0 = __shfl_sync(gmask, rnd.x, ri, G);
            const uint32_t w1 = __shfl_sync(gmask, rnd.y, ri, G);
            const uint32_t w2 = __shfl_sync(gmask, rnd.z, ri, G);
            e1 = -logf(u01_from32(w0));
            u_ev = u01_from64(w1, w2);
        }
        // ---- FP64 scan of the lane sums ----
        double v = static_cast<double>(lsum);
#pragma unroll
        for (int d = 1; d < G; d <<= 1) {
            const double o = __shfl_up_sync(gmask, v, d, G);
            if (g >= d) v += o;
        }
        const double tot = __shfl_sync(gmask, v, G - 1, G);
        if (!(tot > 0.0) || !(tot < 1.0e300)) { status = KMC_ERR_NONFINITE; break; }
        const double target = u_ev * tot;
        const unsigned shift = static_cast<unsigned>(sub * G);
        const unsigned lowG = (G == 32) ? 0xffffffffu : ((1u << G) - 1u);
        const unsigned hitL = (__ballot_sync(gmask, v >= target) >> shift) & lowG;
        const int L = hitL ? (__ffs(hitL) - 1) : (G - 1);
        const double excl = __shfl_up_sync(gmask, v, 1, G);
        const double baseL = __shfl_sync(gmask, g == 0 ? 0.0 : excl, L, G);
        float rem = static_cast<float>(target - baseL);
        // ---- re-evaluate lane L's run and find the event ----
        int chosen = -1, last_pos = -1;
        {
            const int kb = L * M;
            const int ke = min(kb + M, A);
            for (int kc = kb; kc < ke; kc += G) {
                const int k = kc + g;
                float r = 0.0f;
                if (k < ke) {
                    int row, col;
                    decode_pair(k, h, A1, T1, T2, inv1, inv2, row, col);
                    r = pair_rate(tab, S, sm.src[row], sm.tgt[col], cs);
                }
                float q = r;
#pragma unroll
                for (int d = 1; d < G; d <<= 1) {
                    const float o = __shfl_up_sync(gmask, q, d, G);
                    if (g >= d) q += o;
                }
                const bool pos = (k < ke) && (r > 0.0f);
                const unsigned hit = (__ballot_sync(gmask, pos && q >= rem) >> shift) & lowG;
                const unsigned pm = (__ballot_sync(gmask, pos) >> shift) & lowG;
                if (hit) { chosen = kc + __ffs(hit) - 1; break; }
                if (pm) last_pos = kc + 31 - __clz(pm);
                rem -= __shfl_sync(gmask, q, G - 1, G);
            }
        }
        if (chosen < 0) chosen = last_pos;
        if (chosen < 0) { status = KMC_ERR_NONFINITE; break; }
        int row, col;
        decode_pair(chosen, h, A1, T1, T2, inv1, inv2, row, col);
        const int from = sm.src[row].x;
        const int to = sm.tgt[col].x;
        // ---- clock ----
        const float dt = e1 * __frcp_rn(static_cast<float>(tot));
        const double t_before = t;
        t += static_cast<double>(dt);
        __syncwarp(gmask);   // all lanes done reading the lists
        // ---- apply the hop ----
        const bool fa = from < N, tb = to < N;
        for (int j = g; j < N; j += G) {
            float Ej = sm.E[j];
            if (fa && j != from) Ej -= __ldg(&tab[j * S + from]).y;
            if (tb && j != to) Ej += __ldg(&tab[j * S + to]).y;
            sm.E[j] = Ej;
        }
        if (g == 0) {
            if (fa) sm.occw[from >> 5] &= ~(1u << (from & 31));
            else sm.eo[from - N] -= 1;
            if (tb) sm.occw[to >> 5] |= 1u << (to & 31);
            else sm.eo[to - N] += 1;
            if (record) {
                traffic[from * S + to] += 1;
                if (record == KMC_RECORD_GO) traffic[to * S + from] -= 1;
                const double tx = (record == KMC_RECORD_GO) ? t : t_before;
                if (fa) occ_time[from] += tx - occ_since[from];
                if (tb) occ_since[to] = tx;
            }
        }
        h += (tb ? 1 : 0) - (fa ? 1 : 0);
        ++hop;
        __syncwarp(gmask);
    }

    // ---- write back ----
    if (record) {
        for (int j = g; j < N; j += G)
            if ((sm.occw[j >> 5] >> (j & 31)) & 1u) {
                occ_time[j] += t - occ_since[j];
                occ_since[j] = t;
            }
    }
    for (int j = g; j < N; j += G) occ_g[j] = static_cast<uint8_t>((sm.occw[j >> 5] >> (j & 31)) & 1u);
    for (int e = g; e < P; e += G) B.electrode_occupation[eoff + e] += sm.eo[e];
    if (g == 0) {
        B.time[c] = t;
        B.hops_done[c] = hop;
        B.status[c] = status;
        if (B.n_pairs) B.n_pairs[c] += pairs;
    }
}

template <int G>
int launch(const kmc_batch &b, cudaStream_t st)
{
    constexpr int CPW = 32 / G;
    const int wpb = b.warps_per_block;
    const size_t smem = static_cast<size_t>(wpb) * CPW * chain_smem_words(b.max_sites) * 4;
    if (smem > 227 * 1024) return fail(KMC_ERR_INVALID, "engine: %zu bytes of shared memory per block (max_sites %d, G %d, %d warps) exceeds 227 KB", smem, b.max_sites, G, wpb);
    // Raise the dynamic shared-memory limit only when a launch needs more than
    // any before it, so launches under stream capture make no attribute calls
    // once a first launch has run.
    static int configured = 0;
    cudaError_t e;
    if (static_cast<int>(smem) > configured) {
        e = cudaFuncSetAttribute(f32_engine_kernel<G>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(smem));
        if (e != cudaSuccess) return fail_cuda(e, "cudaFuncSetAttribute(engine)");
        configured = static_cast<int>(smem);
    }
    const int grid = (b.n_work + wpb - 1) / wpb;
    if (grid <= 0) return KMC_OK;
    f32_engine_kernel<G><<<grid, wpb * 32, smem, st>>>(b);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail_cuda(e, "engine launch");
    return KMC_OK;
}

}  // namespace

int run_batch(const kmc_batch &b, cudaStream_t st)
{
    if (b.n_chains < 0 || b.n_work < 0 || b.max_sites <= 0 || b.max_sites > kMaxSitesF32)
        return fail(KMC_ERR_INVALID, "engine: bad sizes (n_chains %d, n_work %d, max_sites %d)",
                    b.n_chains, b.n_work, b.max_sites);
    if (b.warps_per_block < 1 || b.warps_per_block > 8)
        return fail(KMC_ERR_INVALID, "engine: warps_per_block %d not in 1..8", b.warps_per_block);
    if (b.max_hops_per_launch <= 0)
        return fail(KMC_ERR_INVALID, "engine: max_hops_per_launch must be positive");
    if (b.record < 0 || b.record > 2) return fail(KMC_ERR_INVALID, "engine: bad record mode %d", b.record);
    if (b.record && (!b.occ_time || !b.occ_since || !b.traffic || !b.chain_pair_off))
        return fail(KMC_ERR_INVALID, "engine: record needs occ_time, occ_since, traffic, chain_pair_off");
    if (!b.tab_N || !b.tab_P || !b.tab_off || !b.tab_LB || !b.chain_tab || !b.chain_kT ||
        !b.chain_site_off || !b.chain_el_off || !b.E_constant || !b.el_energy || !b.occupation ||
        !b.electrode_occupation || !b.time || !b.hops_done || !b.hops_total || !b.stream ||
        !b.status || !b.work)
        return fail(KMC_ERR_INVALID, "engine: a required pointer is NULL");
    if (b.replay && !b.replay_off) return fail(KMC_ERR_INVALID, "engine: replay needs replay_off");
    switch (b.lanes_per_chain) {
    case 4: return launch<4>(b, st);
    case 8: return launch<8>(b, st);
    case 16: return launch<16>(b, st);
    case 32: return launch<32>(b, st);
    default: return fail(KMC_ERR_INVALID, "engine: lanes_per_chain %d not in {4,8,16,32}", b.lanes_per_chain);
    }
}

int engine_smem_words(int max_sites) { return chain_smem_words(max_sites); }

}  // namespace kmc
