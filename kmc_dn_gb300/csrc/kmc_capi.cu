// kmc_capi.cu -- extern "C" entry points (include/kmc_dn_gb300.h).
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
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

// Automatic lanes-per-chain: enough lanes that a chain's pair loop stays
// short, few enough that per-hop group overhead (scans, FP64 compare) is
// shared by several chains per warp.
// Threads per chain by network size, as measured best on GB300: warp
// slices for small networks, whole blocks for large ones.
static int auto_lanes(int S)
{
    if (S <= 48) return 16;
    if (S <= 128) return 32;
    if (S <= 512) return 128;
    return 256;
}

int host_run(const HostRun &h)
{
    const int32_t n_geoms = h.n_geoms;
    const int32_t *geom_N = h.geom_N, *geom_P = h.geom_P;
    const double *geom_nu = h.geom_nu, *geom_I0 = h.geom_I0, *geom_R = h.geom_R;
    const int64_t *geom_pair_off = h.geom_pair_off;
    const double *distances = h.distances, *transitions_constant = h.transitions_constant;
    const int32_t n_chains = h.n_chains;
    const int32_t *chain_geom = h.chain_geom;
    const double *chain_kT = h.chain_kT, *E_constant = h.E_constant, *site_energies_in = h.site_energies;
    uint8_t *occupation = h.occupation;
    const int64_t *hops = h.hops;
    const uint64_t seed = h.seed;
    const int32_t lanes_per_chain = h.lanes_per_chain;
    double *time_out = h.time_out;
    int64_t *electrode_occupation = h.electrode_occupation;
    int32_t *status = h.status;
    const int record = h.record;
    if (n_geoms <= 0 || n_chains < 0) return fail(KMC_ERR_INVALID, "run_batch_host: bad counts");
    if (!geom_N || !geom_P || !geom_nu || !geom_I0 || !geom_R || !geom_pair_off || !distances ||
        !transitions_constant || (n_chains > 0 && (!chain_geom || !chain_kT || !E_constant ||
        !site_energies_in || !occupation || !hops || !time_out || !electrode_occupation || !status)))
        return fail(KMC_ERR_INVALID, "run_batch_host: NULL pointer");
    if (n_chains == 0) return KMC_OK;
    int Smax = 0;
    std::vector<int64_t> tab_off(n_geoms);
    int64_t tab_floats = 0, pair_total = 0;
    for (int g = 0; g < n_geoms; ++g) {
        const int S = geom_N[g] + geom_P[g];
        if (geom_N[g] < 0 || geom_P[g] < 0 || geom_P[g] > 64 || S <= 0 || S > kMaxSitesF32)
            return fail(KMC_ERR_INVALID, "run_batch_host: geometry %d has N=%d P=%d", g, geom_N[g], geom_P[g]);
        tab_off[g] = tab_floats;
        tab_floats += 2 * (int64_t)S * S;
        pair_total = std::max<int64_t>(pair_total, geom_pair_off[g] + (int64_t)S * S);
    }
    std::vector<int64_t> site_off(n_chains), el_off(n_chains), sev_off(n_chains);
    int64_t nsite = 0, nel = 0, nsev = 0, maxhops = 0;
    for (int c = 0; c < n_chains; ++c) {
        const int g = chain_geom[c];
        if (g < 0 || g >= n_geoms) return fail(KMC_ERR_INVALID, "run_batch_host: chain %d geometry %d", c, g);
        if (hops[c] < 0 || !(chain_kT[c] > 0)) return fail(KMC_ERR_INVALID, "run_batch_host: chain %d hops/kT", c);
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
    const int G = lanes_per_chain > 0 ? lanes_per_chain : auto_lanes(Smax);
    if (G != 4 && G != 8 && G != 16 && G != 32 && G != 64 && G != 128 && G != 256 && G != 512)
        return fail(KMC_ERR_INVALID, "run_batch_host: lanes_per_chain %d", G);
    const int CPW = G >= 32 ? 1 : 32 / G;   // chains per warp, or one chain per block
    std::vector<int32_t> order(n_chains);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        const int sa = geom_N[chain_geom[a]] + geom_P[chain_geom[a]];
        const int sb = geom_N[chain_geom[b]] + geom_P[chain_geom[b]];
        if (sa != sb) return sa > sb;
        return hops[a] > hops[b];
    });
    const int n_work = (n_chains + CPW - 1) / CPW;
    std::vector<int32_t> work((size_t)n_work * CPW, -1);
    for (int c = 0; c < n_chains; ++c) work[c] = order[c];
    const int reanchor = 1024;
    int64_t seg = ((maxhops + reanchor - 1) / reanchor) * reanchor;
    if (seg <= 0) seg = reanchor;

    cudaStream_t st;
    cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e != cudaSuccess) return fail_cuda(e, "run_batch_host: stream");
    struct Dev {
        std::vector<void *> ptrs;
        cudaStream_t st;
        ~Dev() {
            for (void *p : ptrs) cudaFreeAsync(p, st);
            cudaStreamSynchronize(st);
            cudaStreamDestroy(st);
        }
    } dev{{}, st};
    auto dalloc = [&](void **p, size_t bytes) -> cudaError_t {
        cudaError_t r = cudaMallocAsync(p, bytes ? bytes : 16, st);
        if (r == cudaSuccess) dev.ptrs.push_back(*p);
        return r;
    };
    auto h2d = [&](void *d, const void *h, size_t bytes) {
        return cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, st);
    };
    double *d_dist = nullptr, *d_tc = nullptr;
    float *d_tab = nullptr, *d_ec = nullptr, *d_vel = nullptr, *d_kT = nullptr;
    int32_t *d_tabN = nullptr, *d_tabP = nullptr, *d_ctab = nullptr, *d_status = nullptr, *d_work = nullptr;
    int64_t *d_taboff = nullptr, *d_soff = nullptr, *d_eoff = nullptr, *d_eo = nullptr;
    int64_t *d_hd = nullptr, *d_ht = nullptr;
    uint8_t *d_occ = nullptr;
    double *d_time = nullptr;
    uint64_t *d_stream = nullptr;
    int64_t *d_poff = nullptr;
    double *d_ot = nullptr, *d_os = nullptr;
    int32_t *d_tr = nullptr;
    std::vector<int64_t> poff(n_chains);
    int64_t npair = 0;
    for (int c = 0; c < n_chains; ++c) {
        const int S = geom_N[chain_geom[c]] + geom_P[chain_geom[c]];
        poff[c] = npair;
        npair += (int64_t)S * S;
    }
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
        (e = dalloc((void **)&d_status, sizeof(int32_t) * n_chains)) != cudaSuccess ||
        (e = dalloc((void **)&d_work, sizeof(int32_t) * work.size())) != cudaSuccess)
        return fail_cuda(e, "run_batch_host: device allocation");
    if (record) {
        if ((e = dalloc((void **)&d_poff, sizeof(int64_t) * n_chains)) != cudaSuccess ||
            (e = dalloc((void **)&d_ot, sizeof(double) * std::max<int64_t>(nsite, 1))) != cudaSuccess ||
            (e = dalloc((void **)&d_os, sizeof(double) * std::max<int64_t>(nsite, 1))) != cudaSuccess ||
            (e = dalloc((void **)&d_tr, sizeof(int32_t) * std::max<int64_t>(npair, 1))) != cudaSuccess)
            return fail_cuda(e, "run_batch_host: record allocation");
        if ((e = h2d(d_poff, poff.data(), sizeof(int64_t) * n_chains)) != cudaSuccess ||
            (e = cudaMemsetAsync(d_ot, 0, sizeof(double) * std::max<int64_t>(nsite, 1), st)) != cudaSuccess ||
            (e = cudaMemsetAsync(d_tr, 0, sizeof(int32_t) * std::max<int64_t>(npair, 1), st)) != cudaSuccess)
            return fail_cuda(e, "run_batch_host: record init");
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
        (e = h2d(d_stream, streams.data(), sizeof(uint64_t) * n_chains)) != cudaSuccess ||
        (e = h2d(d_work, work.data(), sizeof(int32_t) * work.size())) != cudaSuccess)
        return fail_cuda(e, "run_batch_host: copy in");
    if ((e = cudaMemsetAsync(d_eo, 0, sizeof(int64_t) * std::max<int64_t>(nel, 1), st)) != cudaSuccess ||
        (e = cudaMemsetAsync(d_time, 0, sizeof(double) * n_chains, st)) != cudaSuccess ||
        (e = cudaMemsetAsync(d_hd, 0, sizeof(int64_t) * n_chains, st)) != cudaSuccess)
        return fail_cuda(e, "run_batch_host: memset");
    for (int g = 0; g < n_geoms; ++g) {
        const int rc = build_table(geom_N[g], geom_P[g], geom_nu[g], geom_I0[g], geom_R[g],
                                   d_dist + geom_pair_off[g], d_tc + geom_pair_off[g],
                                   d_tab + tab_off[g], st);
        if (rc != KMC_OK) return rc;
    }
    kmc_batch b;
    memset(&b, 0, sizeof(b));
    b.n_tables = n_geoms;
    b.max_sites = Smax;
    b.tab_N = d_tabN;
    b.tab_P = d_tabP;
    b.tab_off = d_taboff;
    b.tab_LB = d_tab;
    b.n_chains = n_chains;
    b.lanes_per_chain = G;
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
    b.work = d_work;
    b.n_work = n_work;
    b.record = record;
    b.chain_pair_off = d_poff;
    b.occ_time = d_ot;
    b.occ_since = d_os;
    b.traffic = d_tr;
    b.reanchor = reanchor;
    b.warps_per_block = 8;
    b.max_hops_per_launch = seg;
    b.seed = seed;
    int rc = run_batch(b, st);
    if (rc != KMC_OK) return rc;
    if ((e = cudaMemcpyAsync(time_out, d_time, sizeof(double) * n_chains, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(electrode_occupation, d_eo, sizeof(int64_t) * nel, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(occupation, d_occ, (size_t)nsite, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(status, d_status, sizeof(int32_t) * n_chains, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return fail_cuda(e, "run_batch_host: copy out");
    std::vector<int32_t> tr_h;
    std::vector<double> ot_h;
    if (record) {
        tr_h.resize(std::max<int64_t>(npair, 1));
        ot_h.resize(std::max<int64_t>(nsite, 1));
        if ((e = cudaMemcpyAsync(tr_h.data(), d_tr, sizeof(int32_t) * tr_h.size(), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
            (e = cudaMemcpyAsync(ot_h.data(), d_ot, sizeof(double) * ot_h.size(), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
            return fail_cuda(e, "run_batch_host: record copy out");
    }
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return fail_cuda(e, "run_batch_host: run");
    if (record) {
        for (int64_t k = 0; k < npair; ++k)
            if (h.traffic_out) h.traffic_out[k] += tr_h[k];
        for (int64_t k = 0; k < nsite; ++k)
            if (h.occ_time_out) h.occ_time_out[k] += ot_h[k];
    }
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
    return (1 << 2) | (1 << 3) | (1 << 4) | (1 << 5);   // bit k set: G = 2^k is compiled in
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

}  // extern "C"
