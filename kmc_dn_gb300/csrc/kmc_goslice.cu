// kmc_goslice.cu -- the Go library's exports (include/kmc_goslice_compat.h)
// on top of the batched engine's host-buffer runner.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstring>
#include <vector>

#include "../../include/kmc_goslice_compat.h"
#include "kmc_internal.h"

namespace {

// The Go library draws from math/rand's global source and is never seeded
// by the caller; each call here takes a fresh seed from a process counter
// mixed with the start time.
uint64_t next_seed()
{
    static std::atomic<uint64_t> counter{0};
    static const uint64_t t0 = static_cast<uint64_t>(
        std::chrono::steady_clock::now().time_since_epoch().count());
    return t0 * 0x9E3779B97F4A7C15ULL + (++counter) * 0xD1B54A32D192ED03ULL;
}

double single_chain(int64_t NSites, int64_t NElectrodes, double prune, double nu, double kT,
                    double I_0, double R, GoSlice distances, GoSlice E_constant,
                    GoSlice transitions_constant, GoSlice electrode_occupation,
                    GoSlice site_energies, int hops, bool record, GoSlice traffic,
                    GoSlice average_occupation)
{
    using namespace kmc;
    const int N = static_cast<int>(NSites), P = static_cast<int>(NElectrodes);
    const int64_t S = (int64_t)N + P;
    if (N < 0 || P < 0 || S <= 0 || hops < 0 || distances.len < S * S ||
        transitions_constant.len < S * S || E_constant.len < N || site_energies.len < S ||
        electrode_occupation.len < P ||
        (record && (traffic.len < S * S || average_occupation.len < N)))
        return fail(KMC_ERR_INVALID, "Go-compatible call: slice lengths do not match N=%d P=%d", N, P);
    std::vector<double> tc(transitions_constant.data, transitions_constant.data + S * S);
    if (prune > 0) {
        // simulation.go:199-215 keeps the pairs with tc > cut * max(tc), all
        // three in float32 (the wrapper converts the tables and the cut to
        // float32 first, simulationWrapper.go:37-56, :98-110); the product is
        // rounded to float32 before the compare.
        float mx = 0.0f;
        for (double x : tc) mx = std::max(mx, static_cast<float>(x));
        const float cut = static_cast<float>(static_cast<float>(prune) * mx);
        for (double &x : tc)
            if (!(static_cast<float>(x) > cut)) x = 0.0;
    }
    const int32_t gN = N, gP = P;
    const int64_t off = 0;
    const int32_t cg = 0;
    std::vector<uint8_t> occ(std::max(N, 1), 0);   // the Go wrappers start empty
    const int64_t h = hops;
    double t = 0.0;
    std::vector<int64_t> eo(std::max(P, 1), 0);
    int32_t st = 0;
    HostRun run;
    memset(&run, 0, sizeof(run));
    run.n_geoms = 1;
    run.geom_N = &gN;
    run.geom_P = &gP;
    run.geom_nu = &nu;
    run.geom_I0 = &I_0;
    run.geom_R = &R;
    run.geom_pair_off = &off;
    run.distances = distances.data;
    run.transitions_constant = tc.data();
    run.n_chains = 1;
    run.chain_geom = &cg;
    run.chain_kT = &kT;
    run.E_constant = E_constant.data;
    run.site_energies = site_energies.data;
    run.occupation = occ.data();
    run.hops = &h;
    run.seed = next_seed();
    run.record = record ? KMC_RECORD_GO : KMC_RECORD_NONE;
    run.time_out = &t;
    run.electrode_occupation = eo.data();
    run.status = &st;
    run.traffic_out = record ? traffic.data : nullptr;
    run.occ_time_out = record ? average_occupation.data : nullptr;
    const int rc = host_run(run);
    if (rc != KMC_OK) return rc;
    if (st != KMC_OK) return fail(st, "Go-compatible call: chain stopped (no allowed transition)");
    for (int e = 0; e < P; ++e) electrode_occupation.data[e] = static_cast<double>(eo[e]);
    return t;
}

}  // namespace

extern "C" {

double wrapperSimulate(int64_t NSites, int64_t NElectrodes, double nu, double kT, double I_0,
                       double R, GoSlice occupation, GoSlice distances, GoSlice E_constant,
                       GoSlice transitions_constant, GoSlice electrode_occupation,
                       GoSlice site_energies, int hops, uint8_t record, GoSlice traffic,
                       GoSlice average_occupation)
{
    (void)occupation;
    return single_chain(NSites, NElectrodes, 0.0, nu, kT, I_0, R, distances, E_constant,
                        transitions_constant, electrode_occupation, site_energies, hops, record != 0,
                        traffic, average_occupation);
}

double wrapperSimulateRecord(int64_t NSites, int64_t NElectrodes, double nu, double kT, double I_0,
                             double R, GoSlice occupation, GoSlice distances, GoSlice E_constant,
                             GoSlice transitions_constant, GoSlice electrode_occupation,
                             GoSlice site_energies, int hops, uint8_t record, GoSlice traffic,
                             GoSlice average_occupation)
{
    (void)occupation;
    return single_chain(NSites, NElectrodes, 0.0, nu, kT, I_0, R, distances, E_constant,
                        transitions_constant, electrode_occupation, site_energies, hops, record != 0,
                        traffic, average_occupation);
}

double wrapperSimulateRecordPlus(int64_t NSites, int64_t NElectrodes, double nu, double kT,
                                 double I_0, double R, GoSlice occupation, GoSlice distances,
                                 GoSlice E_constant, GoSlice transitions_constant,
                                 GoSlice electrode_occupation, GoSlice site_energies, int hops,
                                 uint8_t record, GoSlice traffic, GoSlice average_occupation)
{
    (void)occupation;
    (void)record;
    return single_chain(NSites, NElectrodes, 0.0, nu, kT, I_0, R, distances, E_constant,
                        transitions_constant, electrode_occupation, site_energies, hops, false,
                        traffic, average_occupation);
}

double wrapperSimulatePruned(int64_t NSites, int64_t NElectrodes, double prune_threshold, double nu,
                             double kT, double I_0, double R, GoSlice occupation, GoSlice distances,
                             GoSlice E_constant, GoSlice transitions_constant,
                             GoSlice electrode_occupation, GoSlice site_energies, int hops,
                             uint8_t record, GoSlice traffic, GoSlice average_occupation)
{
    (void)occupation;
    return single_chain(NSites, NElectrodes, prune_threshold, nu, kT, I_0, R, distances, E_constant,
                        transitions_constant, electrode_occupation, site_energies, hops, record != 0,
                        traffic, average_occupation);
}

double wrapperSimulateProbability(int64_t NSites, int64_t NElectrodes, double nu, double kT,
                                  double I_0, double R, GoSlice occupation, GoSlice distances,
                                  GoSlice E_constant, GoSlice transitions_constant,
                                  GoSlice electrode_occupation, GoSlice site_energies, int hops,
                                  uint8_t record, GoSlice traffic, GoSlice average_occupation)
{
    using namespace kmc;
    const int N = static_cast<int>(NSites), P = static_cast<int>(NElectrodes);
    const int64_t S = (int64_t)N + P;
    if (N < 0 || P < 0 || S <= 0 || hops < 0 || occupation.len < N || distances.len < S * S ||
        transitions_constant.len < S * S || E_constant.len < N || site_energies.len < S ||
        electrode_occupation.len < P || (record && (traffic.len < S * S || average_occupation.len < N)))
        return fail(KMC_ERR_INVALID, "wrapperSimulateProbability: slice lengths do not match N=%d P=%d", N, P);
    if (S > kmc_mf_max_sites(KMC_MF_RATES_F64))
        return fail(KMC_ERR_INVALID, "wrapperSimulateProbability: %lld sites exceed the limit %d",
                    (long long)S, kmc_mf_max_sites(KMC_MF_RATES_F64));
    // segments of S entries (simulationWrapper.go:229-232 sets every acceptor to 0.5)
    std::vector<double> occ(S, 0.0), ec(S, 0.0), se(site_energies.data, site_energies.data + S), avg(S, 0.0);
    for (int i = 0; i < N; ++i) { occ[i] = 0.5; ec[i] = E_constant.data[i]; }
    if (record) for (int i = 0; i < N; ++i) avg[i] = average_occupation.data[i];
    std::vector<double> eo(std::max(P, 1), 0.0);
    const int32_t n32 = N, p32 = P;
    const int64_t zero = 0, h = hops;
    double t = 0.0;
    int32_t st = 0;
    int64_t done = 0;
    kmc_mf_batch b;
    memset(&b, 0, sizeof(b));
    b.n_chains = 1;
    b.max_sites = static_cast<int32_t>(S);
    b.rates = KMC_MF_RATES_F64;
    b.record = record ? 1 : 0;
    b.N = &n32; b.P = &p32; b.nu = &nu; b.kT = &kT; b.I_0 = &I_0; b.R = &R;
    b.pair_off = &zero; b.distances = distances.data; b.transitions_constant = transitions_constant.data;
    b.site_off = &zero; b.E_constant = ec.data(); b.site_energies = se.data(); b.occupation = occ.data();
    b.el_off = &zero; b.electrode_occupation = eo.data(); b.hops = &h;
    b.traffic_off = &zero; b.traffic = record ? traffic.data : nullptr;
    b.average_occupation = record ? avg.data() : nullptr;
    b.time = &t; b.status = &st; b.iterations_done = &done;
    const int rc = kmc_mf_run_host(&b, nullptr);
    if (rc != KMC_OK) return rc;
    if (st != KMC_OK) return fail(st, "wrapperSimulateProbability: total rate zero or non-finite");
    for (int i = 0; i < N; ++i) { occupation.data[i] = occ[i]; site_energies.data[i] = se[i]; }
    for (int e = 0; e < P; ++e) electrode_occupation.data[e] = eo[e];
    if (record) for (int i = 0; i < N; ++i) average_occupation.data[i] = avg[i];
    return t;
}

int64_t parallelSimulations(GoSlice NSites, GoSlice NElectrodes, GoSlice nu, GoSlice kT,
                            GoSlice I_0, GoSlice R, GoSlice occupation, GoSlice distances,
                            GoSlice E_constant, GoSlice transitions_constant,
                            GoSlice electrode_occupation, GoSlice hops, GoSlice time,
                            GoSlice site_energies)
{
    using namespace kmc;
    const int64_t n = NSites.len;
    if (n <= 0) return 0;
    if (NElectrodes.len < n || nu.len < n || kT.len < n || I_0.len < n || R.len < n ||
        hops.len < n || time.len < n)
        return fail(KMC_ERR_INVALID, "parallelSimulations: per-chain slices shorter than NSites");
    std::vector<int32_t> gN(n), gP(n), cg(n);
    std::vector<int64_t> poff(n), h(n);
    std::vector<uint8_t> occ;
    int64_t pairs = 0, sites = 0, els = 0, sev = 0;
    for (int64_t c = 0; c < n; ++c) {
        gN[c] = static_cast<int32_t>(NSites.data[c]);
        gP[c] = static_cast<int32_t>(NElectrodes.data[c]);
        cg[c] = static_cast<int32_t>(c);
        h[c] = static_cast<int64_t>(hops.data[c]);
        poff[c] = pairs;
        const int64_t S = (int64_t)gN[c] + gP[c];
        pairs += S * S;
        sites += gN[c];
        els += gP[c];
        sev += S;
    }
    if (occupation.len < sites || distances.len < pairs || transitions_constant.len < pairs ||
        E_constant.len < sites || electrode_occupation.len < els || site_energies.len < sev)
        return fail(KMC_ERR_INVALID, "parallelSimulations: ragged slices shorter than the chains need");
    occ.resize(std::max<int64_t>(sites, 1));
    for (int64_t k = 0; k < sites; ++k) occ[k] = occupation.data[k] > 0 ? 1 : 0;   // simulationWrapper.go:253-259
    std::vector<int64_t> eo(std::max<int64_t>(els, 1), 0);
    std::vector<int32_t> st(n, 0);
    HostRun run;
    memset(&run, 0, sizeof(run));
    run.n_geoms = static_cast<int32_t>(n);
    run.geom_N = gN.data();
    run.geom_P = gP.data();
    run.geom_nu = nu.data;
    run.geom_I0 = I_0.data;
    run.geom_R = R.data;
    run.geom_pair_off = poff.data();
    run.distances = distances.data;
    run.transitions_constant = transitions_constant.data;
    run.n_chains = static_cast<int32_t>(n);
    run.chain_geom = cg.data();
    run.chain_kT = kT.data;
    run.E_constant = E_constant.data;
    run.site_energies = site_energies.data;
    run.occupation = occ.data();
    run.hops = h.data();
    run.seed = next_seed();
    run.time_out = time.data;
    run.electrode_occupation = eo.data();
    run.status = st.data();
    const int rc = host_run(run);
    if (rc != KMC_OK) return rc;
    for (int64_t k = 0; k < els; ++k) electrode_occupation.data[k] = static_cast<double>(eo[k]);
    for (int64_t c = 0; c < n; ++c)
        if (st[c] != KMC_OK) return fail(st[c], "parallelSimulations: chain %lld stopped", (long long)c);
    return 0;
}

int64_t kmc_goslice_abi_probe(GoSlice s0, GoSlice s1, GoSlice s2, GoSlice s3, GoSlice s4,
                              GoSlice s5, GoSlice s6, GoSlice s7, GoSlice s8, GoSlice s9,
                              GoSlice s10, GoSlice s11, GoSlice s12, GoSlice s13)
{
    const GoSlice s[14] = {s0, s1, s2, s3, s4, s5, s6, s7, s8, s9, s10, s11, s12, s13};
    int64_t acc = 0;
    for (int k = 0; k < 14; ++k) acc += (k + 1) * s[k].len;
    return acc;
}

}  // extern "C"
