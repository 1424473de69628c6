// kmc_capi.cu -- extern "C" entry points (include/kmc_dn_gb300.h).
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <numeric>
#include <vector>

#include <cuda_runtime.h>

#include "kmc_internal.h"

namespace kmc {

namespace {
thread_local char g_msg[512] = "";
thread_local int g_code = KMC_OK;
}  // namespace

int fail(int code, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_msg, sizeof(g_msg), fmt, ap);
    va_end(ap);
    g_code = code;
    return code;
}

int fail_cuda(cudaError_t e, const char *what)
{
    const int code = (e == cudaErrorMemoryAllocation) ? KMC_ERR_OOM : KMC_ERR_CUDA;
    return fail(code, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

int ok()
{
    return KMC_OK;
}

// Automatic lanes per chain (threads per chain) by network size, as
// measured best on GB300: enough lanes that a chain's pair walk stays short,
// few enough that the per-hop group work (scan, search, list rebuild) is
// shared by several chains per warp for small networks; whole blocks for
// large ones.
static int auto_lanes(int S)
{
    if (S <= 48) return 16;
    if (S <= 128) return 32;
    if (S <= 512) return 128;
    return 256;
}

// A batch of chains resident on the device: tables, per-chain state and the
// launch description, advanced by run() any number of times (a run split
// into launches gives the results of one launch: quanta start at multiples
// of the re-anchor period and the random streams are counter-based).
struct EngineState {
    cudaStream_t st = nullptr;
    bool own_stream = false;
    std::vector<void *> ptrs;
    kmc_batch b;                       // shared pools; lanes/work/max_sites per bin below
    // One launch per size class: lanes per chain, its work list and the
    // largest network of the class.  Classes after the first run on their own
    // streams, forked from and joined back to `st` with events.
    struct Bin {
        int32_t lanes = 0, n_work = 0, max_sites = 0;
        int32_t *work = nullptr;
    };
    std::vector<Bin> bins;
    std::vector<cudaStream_t> bin_streams;
    std::vector<cudaEvent_t> bin_events;   // [0] fork, [1 + k] join of bin k + 1
    int32_t n_chains = 0;
    int64_t nsite = 0, nel = 0, npair = 0, maxhops = 0;
    int record = 0;
    std::mutex mu;
    ~EngineState()
    {
        for (void *p : ptrs) cudaFreeAsync(p, st);
        if (st) {
            cudaStreamSynchronize(st);
            if (own_stream) cudaStreamDestroy(st);
        }
        for (cudaStream_t s : bin_streams) cudaStreamDestroy(s);
        for (cudaEvent_t e : bin_events) cudaEventDestroy(e);
    }
};

// Lanes per chain of every chain: the caller's choice for all, or by size.
// Chains are binned by it and ordered inside a bin by size, then hop budget
// (both descending), so that chains sharing a warp have similar per-hop work
// and lifetimes -- the order of the Python Batch's work lists.
// A launch of few chains cannot fill the GPU, and its run time is the
// per-hop latency of one chain: each chain then gets a wider group (one
// N=120 chain takes 2.7 us per hop at 256 lanes, 12.9 us at the size
// default of 32), up to twice the next power of two of its site count and
// 512 lanes, while the launch's chains x lanes stay within a quarter of the
// engine's resident threads (512 per SM).  The Python layer applies the
// same rule (engine.widen_small_launch).
static int widen_small_launch(int G, int S, int n_chains, int sms)
{
    int p = 1;
    while (p < S) p <<= 1;
    const int target = std::min(512, 2 * p);
    const int64_t budget = static_cast<int64_t>(sms) * 512 / 4;
    while (G < target && static_cast<int64_t>(n_chains) * 2 * G <= budget) G *= 2;
    return G;
}

static std::vector<int> chain_lanes(const HostRun &h)
{
    std::vector<int> g(h.n_chains);
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        sms = 0;
    for (int c = 0; c < h.n_chains; ++c) {
        const int geo = h.chain_geom[c];
        const int S = h.geom_N[geo] + h.geom_P[geo];
        g[c] = h.lanes_per_chain > 0 ? h.lanes_per_chain
                                     : widen_small_launch(auto_lanes(S), S, h.n_chains, sms);
    }
    return g;
}

// Warps per block for a warp-slice bin of n_work warp items: the size that
// puts the fewest warps on the busiest SM while every block is resident at
// once at 16 warps per SM (2048 items on 152 SMs: 7 warps, 293 blocks, at
// most 14 warps on an SM, where 8 warps leave 104 SMs with 16 and 48 with
// 8); 8 when no size fits in one wave.
static int balanced_warps_per_block(int n_work)
{
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
        return 8;
    int best = 8, best_load = 0;
    for (int w = 8; w >= 4; --w) {
        const int blocks = (n_work + w - 1) / w;
        if (blocks > (16 / w) * sms) continue;
        const int load = ((blocks + sms - 1) / sms) * w;
        if (best_load == 0 || load < best_load) {
            best_load = load;
            best = w;
        }
    }
    return best;
}

// Every kernel loaded once per device before a host path's first launches
// (its size bins run side by side on their own streams).
static int ensure_preloaded()
{
    int dev = 0;
    const cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail_cuda(e, "cudaGetDevice");
    static std::mutex mu;
    static uint64_t done = 0;
    std::lock_guard<std::mutex> lock(mu);
    if (dev < 64 && ((done >> dev) & 1u)) return KMC_OK;
    const int rc = kmc_preload_kernels();
    if (rc == KMC_OK && dev < 64) done |= 1ull << dev;
    return rc;
}

int engine_create(const HostRun &h, cudaStream_t user_stream, EngineState **out)
{
    *out = nullptr;
    const int32_t n_geoms = h.n_geoms;
    const int32_t *geom_N = h.geom_N, *geom_P = h.geom_P;
    const double *geom_nu = h.geom_nu, *geom_I0 = h.geom_I0, *geom_R = h.geom_R;
    const int64_t *geom_pair_off = h.geom_pair_off;
    const double *distances = h.distances, *transitions_constant = h.transitions_constant;
    const int32_t n_chains = h.n_chains;
    const int32_t *chain_geom = h.chain_geom;
    const double *chain_kT = h.chain_kT, *E_constant = h.E_constant, *site_energies_in = h.site_energies;
    const uint8_t *occupation = h.occupation;
    const int64_t *hops = h.hops;
    const int record = h.record;
    if (n_geoms <= 0 || n_chains <= 0) return fail(KMC_ERR_INVALID, "engine: bad counts");
    if (record < 0 || record > 2) return fail(KMC_ERR_INVALID, "engine: bad record mode %d", record);
    if (!geom_N || !geom_P || !geom_nu || !geom_I0 || !geom_R || !geom_pair_off || !distances ||
        !transitions_constant || !chain_geom || !chain_kT || !E_constant || !site_energies_in ||
        !occupation || !hops)
        return fail(KMC_ERR_INVALID, "engine: NULL pointer");
    int Smax = 0;
    std::vector<int64_t> tab_off(n_geoms);
    int64_t tab_floats = 0, pair_total = 0;
    for (int g = 0; g < n_geoms; ++g) {
        const int S = geom_N[g] + geom_P[g];
        if (geom_N[g] < 0 || geom_P[g] < 0 || geom_P[g] > 64 || S <= 0 || S > kMaxSitesF32)
            return fail(KMC_ERR_INVALID, "engine: geometry %d has N=%d P=%d", g, geom_N[g], geom_P[g]);
        tab_off[g] = tab_floats;
        tab_floats += 2 * (int64_t)S * S;
        pair_total = std::max<int64_t>(pair_total, geom_pair_off[g] + (int64_t)S * S);
    }
    std::vector<int64_t> site_off(n_chains), el_off(n_chains), sev_off(n_chains);
    int64_t nsite = 0, nel = 0, nsev = 0, maxhops = 0;
    for (int c = 0; c < n_chains; ++c) {
        const int g = chain_geom[c];
        if (g < 0 || g >= n_geoms) return fail(KMC_ERR_INVALID, "engine: chain %d geometry %d", c, g);
        if (hops[c] < 0 || !(chain_kT[c] > 0)) return fail(KMC_ERR_INVALID, "engine: chain %d hops/kT", c);
        Smax = std::max(Smax, geom_N[g] + geom_P[g]);
        site_off[c] = nsite;
        el_off[c] = nel;
        sev_off[c] = nsev;
        nsite += geom_N[g];
        nel += geom_P[g];
        nsev += geom_N[g] + geom_P[g];
        maxhops = std::max<int64_t>(maxhops, hops[c]);
    }
    // Host-side staging: FP32 energies, electrode energies, work list.
    std::vector<float> ec32(std::max<int64_t>(nsite, 1)), vel32(std::max<int64_t>(nel, 1)), kT32(n_chains);
    std::vector<int32_t> tabid(n_chains);
    std::vector<uint64_t> streams(n_chains);
    for (int c = 0; c < n_chains; ++c) {
        const int g = chain_geom[c], N = geom_N[g], P = geom_P[g];
        for (int i = 0; i < N; ++i) ec32[site_off[c] + i] = static_cast<float>(E_constant[site_off[c] + i]);
        for (int e = 0; e < P; ++e) vel32[el_off[c] + e] = static_cast<float>(site_energies_in[sev_off[c] + N + e]);
        kT32[c] = static_cast<float>(chain_kT[c]);
        tabid[c] = g;
        streams[c] = h.streams ? h.streams[c] : static_cast<uint64_t>(c);
    }
    const std::vector<int> lanes_of = chain_lanes(h);
    std::vector<int> lane_set(lanes_of);
    std::sort(lane_set.begin(), lane_set.end());
    lane_set.erase(std::unique(lane_set.begin(), lane_set.end()), lane_set.end());
    for (int G : lane_set)
        if (G != 4 && G != 8 && G != 16 && G != 32 && G != 64 && G != 128 && G != 256 && G != 512)
            return fail(KMC_ERR_INVALID, "engine: lanes_per_chain %d", G);
    if (int rc = ensure_preloaded(); rc != KMC_OK) return rc;
    const auto site_count = [&](int c) { return geom_N[chain_geom[c]] + geom_P[chain_geom[c]]; };
    // per bin (ascending lanes): its chains by size then hops, descending,
    // where a warp item holds several chains; by work (hops x S^2, longest
    // first) where an item is one chain, so the longest start in the first
    // wave of blocks
    std::vector<std::vector<int32_t>> bin_work(lane_set.size());
    std::vector<int> bin_smax(lane_set.size(), 0);
    for (size_t k = 0; k < lane_set.size(); ++k) {
        const int G = lane_set[k];
        std::vector<int32_t> order;
        for (int c = 0; c < n_chains; ++c)
            if (lanes_of[c] == G) order.push_back(c);
        const int CPW = G >= 32 ? 1 : 32 / G;   // chains per warp, or one chain per block
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
            const int sa = site_count(a), sb = site_count(b);
            if (CPW == 1) {
                const double wa = static_cast<double>(hops[a]) * sa * sa, wb = static_cast<double>(hops[b]) * sb * sb;
                if (wa != wb) return wa > wb;
            }
            if (sa != sb) return sa > sb;
            return hops[a] > hops[b];
        });
        const size_t n_work = (order.size() + CPW - 1) / CPW;
        bin_work[k].assign(n_work * CPW, -1);
        for (size_t i = 0; i < order.size(); ++i) {
            bin_work[k][i] = order[i];
            bin_smax[k] = std::max(bin_smax[k], site_count(order[i]));
        }
    }
    std::vector<int64_t> poff(n_chains);
    int64_t npair = 0;
    for (int c = 0; c < n_chains; ++c) {
        const int S = geom_N[chain_geom[c]] + geom_P[chain_geom[c]];
        poff[c] = npair;
        npair += (int64_t)S * S;
    }

    EngineState *E = new (std::nothrow) EngineState();
    if (!E) return fail(KMC_ERR_OOM, "engine: host allocation");
    std::unique_ptr<EngineState> guard(E);
    cudaError_t e;
    if (user_stream) {
        E->st = user_stream;
    } else {
        if ((e = cudaStreamCreateWithFlags(&E->st, cudaStreamNonBlocking)) != cudaSuccess)
            return fail_cuda(e, "engine: stream");
        E->own_stream = true;
    }
    cudaStream_t st = E->st;
    auto dalloc = [&](void **p, size_t bytes) -> cudaError_t {
        cudaError_t r = cudaMallocAsync(p, bytes ? bytes : 16, st);
        if (r == cudaSuccess) E->ptrs.push_back(*p);
        return r;
    };
    auto h2d = [&](void *d, const void *hp, size_t bytes) {
        return cudaMemcpyAsync(d, hp, bytes, cudaMemcpyHostToDevice, st);
    };
    double *d_dist = nullptr, *d_tc = nullptr;
    float *d_tab = nullptr, *d_ec = nullptr, *d_vel = nullptr, *d_kT = nullptr;
    int32_t *d_tabN = nullptr, *d_tabP = nullptr, *d_ctab = nullptr, *d_status = nullptr;
    int64_t *d_taboff = nullptr, *d_soff = nullptr, *d_eoff = nullptr, *d_eo = nullptr;
    int64_t *d_hd = nullptr, *d_ht = nullptr;
    uint8_t *d_occ = nullptr;
    double *d_time = nullptr;
    uint64_t *d_stream = nullptr;
    int64_t *d_poff = nullptr;
    double *d_ot = nullptr, *d_os = nullptr;
    int32_t *d_tr = nullptr;
    const size_t pair_bytes = sizeof(double) * (size_t)pair_total;
    if ((e = dalloc((void **)&d_dist, pair_bytes)) != cudaSuccess ||
        (e = dalloc((void **)&d_tc, pair_bytes)) != cudaSuccess ||
        (e = dalloc((void **)&d_tab, sizeof(float) * (size_t)tab_floats)) != cudaSuccess ||
        (e = dalloc((void **)&d_ec, sizeof(float) * ec32.size())) != cudaSuccess ||
        (e = dalloc((void **)&d_vel, sizeof(float) * vel32.size())) != cudaSuccess ||
        (e = dalloc((void **)&d_kT, sizeof(float) * n_chains)) != cudaSuccess ||
        (e = dalloc((void **)&d_tabN, sizeof(int32_t) * n_geoms)) != cudaSuccess ||
        (e = dalloc((void **)&d_tabP, sizeof(int32_t) * n_geoms)) != cudaSuccess ||
        (e = dalloc((void **)&d_taboff, sizeof(int64_t) * n_geoms)) != cudaSuccess ||
        (e = dalloc((void **)&d_ctab, sizeof(int32_t) * n_chains)) != cudaSuccess ||
        (e = dalloc((void **)&d_soff, sizeof(int64_t) * n_chains)) != cudaSuccess ||
        (e = dalloc((void **)&d_eoff, sizeof(int64_t) * n_chains)) != cudaSuccess ||
        (e = dalloc((void **)&d_occ, std::max<int64_t>(nsite, 1))) != cudaSuccess ||
        (e = dalloc((void **)&d_eo, sizeof(int64_t) * std::max<int64_t>(nel, 1))) != cudaSuccess ||
        (e = dalloc((void **)&d_time, sizeof(double) * n_chains)) != cudaSuccess ||
        (e = dalloc((void **)&d_hd, sizeof(int64_t) * n_chains)) != cudaSuccess ||
        (e = dalloc((void **)&d_ht, sizeof(int64_t) * n_chains)) != cudaSuccess ||
        (e = dalloc((void **)&d_stream, sizeof(uint64_t) * n_chains)) != cudaSuccess ||
        (e = dalloc((void **)&d_status, sizeof(int32_t) * n_chains)) != cudaSuccess)
        return fail_cuda(e, "engine: device allocation");
    E->bins.resize(lane_set.size());
    for (size_t k = 0; k < lane_set.size(); ++k) {
        EngineState::Bin &bn = E->bins[k];
        bn.lanes = lane_set[k];
        bn.max_sites = bin_smax[k];
        bn.n_work = static_cast<int32_t>(bin_work[k].size() / (bn.lanes >= 32 ? 1 : 32 / bn.lanes));
        if ((e = dalloc((void **)&bn.work, sizeof(int32_t) * bin_work[k].size())) != cudaSuccess ||
            (e = h2d(bn.work, bin_work[k].data(), sizeof(int32_t) * bin_work[k].size())) != cudaSuccess)
            return fail_cuda(e, "engine: work lists");
    }
    for (size_t k = 1; k < lane_set.size(); ++k) {
        cudaStream_t bs = nullptr;
        if ((e = cudaStreamCreateWithFlags(&bs, cudaStreamNonBlocking)) != cudaSuccess)
            return fail_cuda(e, "engine: bin stream");
        E->bin_streams.push_back(bs);
    }
    for (size_t k = 0; k < lane_set.size(); ++k) {
        cudaEvent_t ev = nullptr;
        if ((e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess)
            return fail_cuda(e, "engine: bin event");
        E->bin_events.push_back(ev);
    }
    if (record) {
        if ((e = dalloc((void **)&d_poff, sizeof(int64_t) * n_chains)) != cudaSuccess ||
            (e = dalloc((void **)&d_ot, sizeof(double) * std::max<int64_t>(nsite, 1))) != cudaSuccess ||
            (e = dalloc((void **)&d_os, sizeof(double) * std::max<int64_t>(nsite, 1))) != cudaSuccess ||
            (e = dalloc((void **)&d_tr, sizeof(int32_t) * std::max<int64_t>(npair, 1))) != cudaSuccess)
            return fail_cuda(e, "engine: record allocation");
        if ((e = h2d(d_poff, poff.data(), sizeof(int64_t) * n_chains)) != cudaSuccess ||
            (e = cudaMemsetAsync(d_ot, 0, sizeof(double) * std::max<int64_t>(nsite, 1), st)) != cudaSuccess ||
            (e = cudaMemsetAsync(d_tr, 0, sizeof(int32_t) * std::max<int64_t>(npair, 1), st)) != cudaSuccess)
            return fail_cuda(e, "engine: record init");
    }
    if ((e = h2d(d_dist, distances, pair_bytes)) != cudaSuccess ||
        (e = h2d(d_tc, transitions_constant, pair_bytes)) != cudaSuccess ||
        (e = h2d(d_ec, ec32.data(), sizeof(float) * ec32.size())) != cudaSuccess ||
        (e = h2d(d_vel, vel32.data(), sizeof(float) * vel32.size())) != cudaSuccess ||
        (e = h2d(d_kT, kT32.data(), sizeof(float) * n_chains)) != cudaSuccess ||
        (e = h2d(d_tabN, geom_N, sizeof(int32_t) * n_geoms)) != cudaSuccess ||
        (e = h2d(d_tabP, geom_P, sizeof(int32_t) * n_geoms)) != cudaSuccess ||
        (e = h2d(d_taboff, tab_off.data(), sizeof(int64_t) * n_geoms)) != cudaSuccess ||
        (e = h2d(d_ctab, tabid.data(), sizeof(int32_t) * n_chains)) != cudaSuccess ||
        (e = h2d(d_soff, site_off.data(), sizeof(int64_t) * n_chains)) != cudaSuccess ||
        (e = h2d(d_eoff, el_off.data(), sizeof(int64_t) * n_chains)) != cudaSuccess ||
        (e = h2d(d_occ, occupation, (size_t)nsite)) != cudaSuccess ||
        (e = h2d(d_ht, hops, sizeof(int64_t) * n_chains)) != cudaSuccess ||
        (e = h2d(d_stream, streams.data(), sizeof(uint64_t) * n_chains)) != cudaSuccess)
        return fail_cuda(e, "engine: copy in");
    if ((e = cudaMemsetAsync(d_eo, 0, sizeof(int64_t) * std::max<int64_t>(nel, 1), st)) != cudaSuccess ||
        (e = cudaMemsetAsync(d_time, 0, sizeof(double) * n_chains, st)) != cudaSuccess ||
        (e = cudaMemsetAsync(d_hd, 0, sizeof(int64_t) * n_chains, st)) != cudaSuccess)
        return fail_cuda(e, "engine: memset");
    for (int g = 0; g < n_geoms; ++g) {
        const int rc = build_table(geom_N[g], geom_P[g], geom_nu[g], geom_I0[g], geom_R[g],
                                   d_dist + geom_pair_off[g], d_tc + geom_pair_off[g],
                                   d_tab + tab_off[g], st);
        if (rc != KMC_OK) return rc;
    }
    // the FP64 source tables are needed only to build the FP32 ones
    // (freed with the engine; stream order keeps them alive for build_table)
    kmc_batch &b = E->b;
    memset(&b, 0, sizeof(b));
    b.n_tables = n_geoms;
    b.max_sites = Smax;
    b.tab_N = d_tabN;
    b.tab_P = d_tabP;
    b.tab_off = d_taboff;
    b.tab_LB = d_tab;
    b.n_chains = n_chains;
    b.chain_tab = d_ctab;
    b.chain_kT = d_kT;
    b.chain_site_off = d_soff;
    b.chain_el_off = d_eoff;
    b.E_constant = d_ec;
    b.el_energy = d_vel;
    b.occupation = d_occ;
    b.electrode_occupation = d_eo;
    b.time = d_time;
    b.hops_done = d_hd;
    b.hops_total = d_ht;
    b.stream = d_stream;
    b.status = d_status;
    b.record = record;
    b.chain_pair_off = d_poff;
    b.occ_time = d_ot;
    b.occ_since = d_os;
    b.traffic = d_tr;
    b.reanchor = 1024;
    // one temperature for every chain: the launch may stage (L, L + c B)
    b.uniform_kT = 0.0f;
    if (n_chains > 0 && std::all_of(kT32.begin(), kT32.end(), [&](float v) { return v == kT32[0]; }))
        b.uniform_kT = kT32[0];
    b.warps_per_block = 8;
    b.max_hops_per_launch = 1024;
    b.seed = h.seed;
    E->n_chains = n_chains;
    E->nsite = nsite;
    E->nel = nel;
    E->npair = npair;
    E->maxhops = maxhops;
    E->record = record;
    *out = guard.release();
    return KMC_OK;
}

// Advance every chain by up to max_hops hops (rounded up to the re-anchor
// period; <= 0: to its budget).  Asynchronous on the engine's stream.
int engine_run(EngineState &E, int64_t max_hops)
{
    const int64_t reanchor = E.b.reanchor;
    int64_t seg = max_hops > 0 ? max_hops : E.maxhops;
    seg = std::max<int64_t>(reanchor, ((seg + reanchor - 1) / reanchor) * reanchor);
    E.b.max_hops_per_launch = seg;
    const size_t nb = E.bins.size();
    cudaError_t e;
    if (nb > 1) {   // fork: the other bins' streams start after the work queued on st
        if ((e = cudaEventRecord(E.bin_events[0], E.st)) != cudaSuccess) return fail_cuda(e, "engine: fork");
        for (size_t k = 1; k < nb; ++k)
            if ((e = cudaStreamWaitEvent(E.bin_streams[k - 1], E.bin_events[0], 0)) != cudaSuccess)
                return fail_cuda(e, "engine: fork");
    }
    for (size_t k = 0; k < nb; ++k) {
        const EngineState::Bin &bn = E.bins[k];
        kmc_batch b = E.b;
        b.lanes_per_chain = bn.lanes;
        b.max_sites = bn.max_sites;
        b.work = bn.work;
        b.n_work = bn.n_work;
        if (bn.lanes <= 32) b.warps_per_block = balanced_warps_per_block(bn.n_work);
        const int rc = run_batch(b, k == 0 ? E.st : E.bin_streams[k - 1]);
        if (rc != KMC_OK) return rc;
    }
    for (size_t k = 1; k < nb; ++k) {   // join back onto st
        if ((e = cudaEventRecord(E.bin_events[k], E.bin_streams[k - 1])) != cudaSuccess ||
            (e = cudaStreamWaitEvent(E.st, E.bin_events[k], 0)) != cudaSuccess)
            return fail_cuda(e, "engine: join");
    }
    return KMC_OK;
}

// Copy results to the host (synchronises the engine's stream).  traffic_out
// (S*S per chain, row-major, chain order) and occ_time_out (N per chain)
// receive the cumulative record-mode sums; any output may be NULL.
int engine_read(EngineState &E, double *time_out, int64_t *electrode_occupation, uint8_t *occupation,
                int32_t *status, int64_t *hops_done, double *traffic_out, double *occ_time_out)
{
    cudaStream_t st = E.st;
    cudaError_t e = cudaSuccess;
    auto d2h = [&](void *hp, const void *d, size_t bytes) {
        if (hp && e == cudaSuccess) e = cudaMemcpyAsync(hp, d, bytes, cudaMemcpyDeviceToHost, st);
    };
    d2h(time_out, E.b.time, sizeof(double) * E.n_chains);
    d2h(electrode_occupation, E.b.electrode_occupation, sizeof(int64_t) * E.nel);
    d2h(occupation, E.b.occupation, (size_t)E.nsite);
    d2h(status, E.b.status, sizeof(int32_t) * E.n_chains);
    d2h(hops_done, E.b.hops_done, sizeof(int64_t) * E.n_chains);
    std::vector<int32_t> tr_h;
    if (E.record && traffic_out) {
        tr_h.resize(std::max<int64_t>(E.npair, 1));
        d2h(tr_h.data(), E.b.traffic, sizeof(int32_t) * tr_h.size());
    }
    if (E.record) d2h(occ_time_out, E.b.occ_time, sizeof(double) * E.nsite);
    if (e != cudaSuccess) return fail_cuda(e, "engine: copy out");
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return fail_cuda(e, "engine: run");
    if (E.record && traffic_out)
        for (int64_t k = 0; k < E.npair; ++k) traffic_out[k] = static_cast<double>(tr_h[k]);
    if (!E.record && occ_time_out) std::fill(occ_time_out, occ_time_out + E.nsite, 0.0);
    return KMC_OK;
}

int host_run(const HostRun &h)
{
    if (h.n_chains == 0) return KMC_OK;
    if (h.n_chains > 0 && (!h.time_out || !h.electrode_occupation || !h.status || !h.occupation))
        return fail(KMC_ERR_INVALID, "run_batch_host: NULL pointer");
    EngineState *E = nullptr;
    int rc = engine_create(h, nullptr, &E);
    if (rc != KMC_OK) return rc;
    std::unique_ptr<EngineState> guard(E);
    if ((rc = engine_run(*E, E->maxhops)) != KMC_OK) return rc;
    std::vector<double> tr, ot;
    if (h.record && h.traffic_out) tr.resize(std::max<int64_t>(E->npair, 1));
    if (h.record && h.occ_time_out) ot.resize(std::max<int64_t>(E->nsite, 1));
    rc = engine_read(*E, h.time_out, h.electrode_occupation, h.occupation, h.status, nullptr,
                     tr.empty() ? nullptr : tr.data(), ot.empty() ? nullptr : ot.data());
    if (rc != KMC_OK) return rc;
    // the record outputs accumulate onto the caller's arrays
    for (int64_t k = 0; k < (int64_t)tr.size() && k < E->npair; ++k) h.traffic_out[k] += tr[k];
    for (int64_t k = 0; k < (int64_t)ot.size() && k < E->nsite; ++k) h.occ_time_out[k] += ot[k];
    return KMC_OK;
}

}  // namespace kmc

using namespace kmc;

extern "C" {

int kmc_version(void)
{
    return 100;   // 0.1.0
}

int kmc_last_error(char *buf, size_t len)
{
    if (buf && len) {
        strncpy(buf, g_msg, len - 1);
        buf[len - 1] = '\0';
    }
    return g_code;
}

int kmc_engine_lane_options(void)
{
    // bit k set: G = 2^k lanes per chain is compiled in (warp slices 4..32,
    // block groups 64..512)
    return (1 << 2) | (1 << 3) | (1 << 4) | (1 << 5) | (1 << 6) | (1 << 7) | (1 << 8) | (1 << 9);
}

int kmc_section_clocks(uint64_t *cycles, int32_t reset)
{
    return kmc::section_clocks(cycles, reset);
}

size_t kmc_simulate_f64_workspace_size(int32_t n_sites)
{
    return n_sites > 0 ? f64_workspace_size(n_sites) : 0;
}

int kmc_simulate_f64(int32_t n_acceptors, int32_t n_electrodes, double nu, double kT, double I_0,
                     double R, uint8_t *occupation, const double *distances,
                     const double *E_constant, const double *site_energies,
                     const double *transitions_constant, int64_t *electrode_occupation,
                     int64_t hops, int32_t record, double *traffic, double *occupations_in_time,
                     const double *uniforms, uint64_t seed, int32_t *hop_log, double *time_out,
                     int32_t *status_out, void *workspace, size_t workspace_bytes, void *stream)
{
    return simulate_f64(n_acceptors, n_electrodes, nu, kT, I_0, R, occupation, distances,
                        E_constant, site_energies, transitions_constant, electrode_occupation,
                        hops, record, traffic, occupations_in_time, uniforms, seed, hop_log,
                        time_out, status_out, workspace, workspace_bytes,
                        static_cast<cudaStream_t>(stream));
}

size_t kmc_simulate_f64_batch_workspace_size(int32_t n_chains, int32_t max_sites)
{
    return (n_chains > 0 && max_sites > 0) ? f64_batch_workspace_size(n_chains, max_sites) : 0;
}

int kmc_simulate_f64_batch(const kmc_f64_batch *batch, void *stream)
{
    if (!batch) return fail(KMC_ERR_INVALID, "kmc_simulate_f64_batch: NULL batch");
    return simulate_f64_batch(*batch, static_cast<cudaStream_t>(stream));
}

int kmc_simulate_f64_flux(int32_t n_acceptors, int32_t n_electrodes, double nu, double kT, double I_0,
                          double R, uint8_t *occupation, const double *distances,
                          const double *E_constant, const double *site_energies,
                          const double *transitions_constant, int64_t *electrode_occupation,
                          int64_t hops, int32_t record, double *traffic, double *occupations_in_time,
                          const double *uniforms, uint64_t seed, int32_t *hop_log, double *time_out,
                          int32_t *status_out, void *workspace, size_t workspace_bytes, void *stream,
                          double *flux_time)
{
    if (!flux_time) return fail(KMC_ERR_INVALID, "kmc_simulate_f64_flux: flux_time is NULL");
    return simulate_f64(n_acceptors, n_electrodes, nu, kT, I_0, R, occupation, distances,
                        E_constant, site_energies, transitions_constant, electrode_occupation,
                        hops, record, traffic, occupations_in_time, uniforms, seed, hop_log,
                        time_out, status_out, workspace, workspace_bytes,
                        static_cast<cudaStream_t>(stream), flux_time);
}

int kmc_build_table(int32_t n_acceptors, int32_t n_electrodes, double nu, double I_0, double R,
                    const double *distances, const double *transitions_constant, float *tab_LB,
                    void *stream)
{
    return build_table(n_acceptors, n_electrodes, nu, I_0, R, distances, transitions_constant,
                       tab_LB, static_cast<cudaStream_t>(stream));
}

int kmc_site_energies(int32_t n_chains, int32_t n_acceptors, int32_t n_electrodes,
                      const double *basis, const double *voltages, double mu, const double *comp,
                      float *E_constant, float *el_energy, void *stream)
{
    return site_energies(n_chains, n_acceptors, n_electrodes, basis, voltages, mu, comp, E_constant,
                         el_energy, static_cast<cudaStream_t>(stream));
}

int kmc_run_batch(const kmc_batch *batch, void *stream)
{
    if (!batch) return fail(KMC_ERR_INVALID, "kmc_run_batch: NULL batch");
    return run_batch(*batch, static_cast<cudaStream_t>(stream));
}

int kmc_run_batch_host(int32_t n_geoms, const int32_t *geom_N, const int32_t *geom_P,
                       const double *geom_nu, const double *geom_I0, const double *geom_R,
                       const int64_t *geom_pair_off, const double *distances,
                       const double *transitions_constant, int32_t n_chains,
                       const int32_t *chain_geom, const double *chain_kT, const double *E_constant,
                       const double *site_energies_in, uint8_t *occupation, const int64_t *hops,
                       uint64_t seed, int32_t lanes_per_chain, double *time_out,
                       int64_t *electrode_occupation, int32_t *status)
{
    HostRun h;
    memset(&h, 0, sizeof(h));
    h.n_geoms = n_geoms;
    h.geom_N = geom_N;
    h.geom_P = geom_P;
    h.geom_nu = geom_nu;
    h.geom_I0 = geom_I0;
    h.geom_R = geom_R;
    h.geom_pair_off = geom_pair_off;
    h.distances = distances;
    h.transitions_constant = transitions_constant;
    h.n_chains = n_chains;
    h.chain_geom = chain_geom;
    h.chain_kT = chain_kT;
    h.E_constant = E_constant;
    h.site_energies = site_energies_in;
    h.occupation = occupation;
    h.hops = hops;
    h.seed = seed;
    h.lanes_per_chain = lanes_per_chain;
    h.time_out = time_out;
    h.electrode_occupation = electrode_occupation;
    h.status = status;
    return host_run(h);
}

int kmc_cancel_word_create(int32_t **host_word, int32_t **device_word)
{
    if (!host_word || !device_word) return fail(KMC_ERR_INVALID, "kmc_cancel_word_create: NULL argument");
    *host_word = nullptr;
    *device_word = nullptr;
    void *h = nullptr, *d = nullptr;
    cudaError_t e = cudaHostAlloc(&h, sizeof(int32_t), cudaHostAllocMapped);
    if (e != cudaSuccess) return fail_cuda(e, "kmc_cancel_word_create: cudaHostAlloc");
    *static_cast<volatile int32_t *>(h) = 0;
    e = cudaHostGetDevicePointer(&d, h, 0);
    if (e != cudaSuccess) {
        cudaFreeHost(h);
        return fail_cuda(e, "kmc_cancel_word_create: cudaHostGetDevicePointer");
    }
    *host_word = static_cast<int32_t *>(h);
    *device_word = static_cast<int32_t *>(d);
    return KMC_OK;
}

void kmc_cancel_word_destroy(int32_t *host_word)
{
    if (host_word) cudaFreeHost(host_word);
}

int kmc_engine_create(kmc_engine **engine, int32_t n_geoms, const int32_t *geom_N, const int32_t *geom_P,
                      const double *geom_nu, const double *geom_I0, const double *geom_R,
                      const int64_t *geom_pair_off, const double *distances,
                      const double *transitions_constant, int32_t n_chains, const int32_t *chain_geom,
                      const double *chain_kT, const double *E_constant, const double *site_energies_in,
                      const uint8_t *occupation, const int64_t *hops, uint64_t seed,
                      int32_t lanes_per_chain, int32_t record, void *stream)
{
    if (!engine) return fail(KMC_ERR_INVALID, "kmc_engine_create: NULL handle pointer");
    *engine = nullptr;
    HostRun h;
    memset(&h, 0, sizeof(h));
    h.n_geoms = n_geoms;
    h.geom_N = geom_N;
    h.geom_P = geom_P;
    h.geom_nu = geom_nu;
    h.geom_I0 = geom_I0;
    h.geom_R = geom_R;
    h.geom_pair_off = geom_pair_off;
    h.distances = distances;
    h.transitions_constant = transitions_constant;
    h.n_chains = n_chains;
    h.chain_geom = chain_geom;
    h.chain_kT = chain_kT;
    h.E_constant = E_constant;
    h.site_energies = site_energies_in;
    h.occupation = const_cast<uint8_t *>(occupation);   // read only here
    h.hops = hops;
    h.seed = seed;
    h.lanes_per_chain = lanes_per_chain;
    h.record = record;
    EngineState *E = nullptr;
    const int rc = engine_create(h, static_cast<cudaStream_t>(stream), &E);
    if (rc == KMC_OK) *engine = reinterpret_cast<kmc_engine *>(E);
    return rc;
}

int kmc_engine_run(kmc_engine *engine, int64_t max_hops)
{
    if (!engine) return fail(KMC_ERR_INVALID, "kmc_engine_run: NULL engine");
    EngineState *E = reinterpret_cast<EngineState *>(engine);
    std::lock_guard<std::mutex> lock(E->mu);
    return engine_run(*E, max_hops);
}

int kmc_engine_read(kmc_engine *engine, double *time_out, int64_t *electrode_occupation, uint8_t *occupation,
                    int32_t *status, int64_t *hops_done, double *traffic, double *occupations_in_time)
{
    if (!engine) return fail(KMC_ERR_INVALID, "kmc_engine_read: NULL engine");
    EngineState *E = reinterpret_cast<EngineState *>(engine);
    std::lock_guard<std::mutex> lock(E->mu);
    return engine_read(*E, time_out, electrode_occupation, occupation, status, hops_done, traffic,
                       occupations_in_time);
}

void kmc_engine_destroy(kmc_engine *engine)
{
    delete reinterpret_cast<EngineState *>(engine);
}

int kmc_preload_kernels(void)
{
    int rc;
    if ((rc = kmc::preload_warp_table()) != KMC_OK) return rc;
    if ((rc = kmc::preload_warp_positions()) != KMC_OK) return rc;
    if ((rc = kmc::preload_block()) != KMC_OK) return rc;
    if ((rc = kmc::preload_f64()) != KMC_OK) return rc;
    if ((rc = kmc::preload_setup()) != KMC_OK) return rc;
    if ((rc = kmc::preload_meanfield()) != KMC_OK) return rc;
    if ((rc = kmc::preload_laplace()) != KMC_OK) return rc;
    return kmc::ok();
}

}  // extern "C"
