/*
 * kmc_oracle.c -- CPU restatement of the reference's hop loops.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle the CUDA kernels are
 * checked against (tests/, __graft_entry__.smoke) and the timed CPU
 * baseline of bench.py; the product path never links or calls it.
 *
 * Two loops are restated:
 *
 *  oracle_numba_replay  -- _simulate_discrete_record, kmc_dopant_networks.py:33-135,
 *                          FP64, fed from an injected uniform stream (two per
 *                          hop: clock, then event).  Every expression keeps the
 *                          reference's operand order so that the FP64 values
 *                          agree to the last bit where libm agrees:
 *                            energies  :59-66   E_i = Ec_i + (-I_0*R)*sum_j (1-occ_j)/d_ij
 *                            rates     :69-87   tc_ij * (dE>0 ? nu*exp(-dE/kT) : nu)
 *                            predicate :137-163
 *                            cumsum    :91-97   row-major, sequential
 *                            clock     :100     -log(1-u) * (1/total)
 *                            select    :103-110 first k with cum_k/total >= u
 *                            hop       :116-123, record :126-130 (post-hop credit)
 *
 *  oracle_go_simulate   -- Go simulate() with wrapperSimulate semantics and no
 *                          state memo, goSimulation/simulation.go:194-325:
 *                          FP32 tables/energies/rates (calcTransitionList :58-80),
 *                          O(N) incremental energies (makeJump :107-130),
 *                          FP32 cumulative list (:270-276), FP64 clock (:297-298),
 *                          halving search (getRandomEvent :163-188), net
 *                          traffic and pre-hop occupancy credit (:309-317).
 *                          Go's math/rand is replaced by a counter-based
 *                          generator (SplitMix64); results agree statistically.
 *
 *  oracle_prob_simulate -- Go probSimulate, the mean-field relaxation of
 *                          goSimulation/probabilitySimulation.go:53-157, FP64,
 *                          every accumulation in the Go loop order (rates
 *                          calcProbTransitions :7-35, step :95-110, apply
 *                          :118-142, clamp :143-152).
 *
 * Parity of oracle_numba_replay is pinned by tests/golden (hop sequences of
 * the reference's own function, run in plain Python with a replay stream).
 * oracle_prob_simulate has no golden vectors (the Go toolchain is absent);
 * it is pinned by the closed-form single-site case, where the mean-field
 * equation is exact.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* ----------------------------------------------------------------------- */
/* numba-path restatement                                                    */
/* ----------------------------------------------------------------------- */

static int possible(int i, int j, int N, const uint8_t *occ)
{
    /* _transition_possible, kmc_dopant_networks.py:137-163 */
    if (i >= N && j >= N) return 0;
    if (i >= N) return occ[j] ? 0 : 1;
    if (j >= N) return occ[i] ? 1 : 0;
    if (i == j) return 0;
    return (!occ[i] || occ[j]) ? 0 : 1;
}

/* Energies (into se, first N entries) and the row-major cumulative rates
 * (into cum, S*S entries) of one state, kmc_dopant_networks.py:59-97, every
 * expression in the reference's operand order.  Returns the total rate. */
static double numba_state_rates(int N, int P, double nu, double kT, double I_0, double R,
                                const uint8_t *occupation, const double *distances,
                                const double *E_constant, const double *transitions_constant,
                                double *se, double *cum)
{
    const int S = N + P;
    const double mIR = -I_0 * R;   /* -I_0*R, evaluated left to right */
    const double IR = I_0 * R;
    for (int i = 0; i < N; ++i) {
        double acc = 0.0;
        for (int j = 0; j < N; ++j)
            if (j != i) acc += (double)(1 - occupation[j]) / distances[(size_t)i * S + j];
        se[i] = E_constant[i];
        se[i] += mIR * acc;
    }
    double run = 0.0;
    for (int i = 0; i < S; ++i) {
        for (int j = 0; j < S; ++j) {
            double t;
            if (!possible(i, j, N, occupation)) {
                t = 0.0;
            } else {
                double dE;
                if (i < N && j < N)
                    dE = se[j] - se[i] - IR / distances[(size_t)i * S + j];
                else
                    dE = se[j] - se[i];
                t = (dE > 0) ? nu * exp(-dE / kT) : nu;
            }
            t = transitions_constant[(size_t)i * S + j] * t;
            size_t k = (size_t)i * S + j;
            run = (k == 0) ? t : t + run;
            cum[k] = run;
        }
    }
    return cum[(size_t)S * S - 1];
}

/* First pair k with cum_k/total >= u (kmc_dopant_networks.py:103-110), and
 * the distance of u from that pair's two cumulative boundaries as a
 * fraction of the total rate. */
static size_t numba_select(const double *cum, size_t SS, double total, double u, double *margin)
{
    size_t ev = 0;
    for (size_t k = 0; k < SS; ++k) {
        if (cum[k] / total >= u) { ev = k; break; }
    }
    if (margin) {
        const double hi = cum[ev] / total - u;
        const double lo = u - (ev > 0 ? cum[ev - 1] / total : 0.0);
        *margin = hi < lo ? hi : lo;
    }
    return ev;
}

/* Returns 0 on success, -1 on bad arguments, -2 on allocation failure.
 * occupation (N, in/out), electrode_occupation (P, in/out) as in the
 * reference; traffic (S*S) and occupations_in_time (N) are accumulated when
 * record != 0 (pass zeroed buffers); hop_log (2*hops), hop_times (hops),
 * margins (hops: distance of the event uniform from the chosen pair's
 * cumulative boundaries, relative to the total rate), hop_totals (hops: the
 * total rate) and hop_rates (hops: the chosen pair's rate) are optional. */
int oracle_numba_replay(int N, int P, double nu, double kT, double I_0, double R,
                        uint8_t *occupation, const double *distances,
                        const double *E_constant, const double *site_energies_in,
                        const double *transitions_constant, int64_t *electrode_occupation,
                        int64_t hops, int record, const double *uniforms,
                        double *time_out, double *traffic, double *occupations_in_time,
                        int32_t *hop_log, double *hop_times, double *margins,
                        double *hop_totals, double *hop_rates)
{
    const int S = N + P;
    if (N < 0 || P < 0 || S <= 0 || hops < 0 || !uniforms || !time_out) return -1;
    double *se = (double *)malloc(sizeof(double) * (size_t)S);
    double *cum = (double *)malloc(sizeof(double) * (size_t)S * (size_t)S);
    if (!se || !cum) { free(se); free(cum); return -2; }
    memcpy(se, site_energies_in, sizeof(double) * (size_t)S);
    double time = 0.0;
    for (int64_t hop = 0; hop < hops; ++hop) {
        const double total = numba_state_rates(N, P, nu, kT, I_0, R, occupation, distances, E_constant,
                                               transitions_constant, se, cum);
        const double scale = 1.0 / total;
        const double u1 = uniforms[2 * hop], u2 = uniforms[2 * hop + 1];
        const double hop_time = -log(1.0 - u1) * scale;
        double mg = 0.0;
        const size_t ev = numba_select(cum, (size_t)S * S, total, u2, &mg);
        if (margins) margins[hop] = mg;
        if (hop_totals) hop_totals[hop] = total;
        if (hop_rates) hop_rates[hop] = cum[ev] - (ev > 0 ? cum[ev - 1] : 0.0);
        int from = (int)(ev / (size_t)S), to = (int)(ev % (size_t)S);
        if (from < N) occupation[from] = 0; else electrode_occupation[from - N] -= 1;
        if (to < N) occupation[to] = 1; else electrode_occupation[to - N] += 1;
        if (record) {
            traffic[(size_t)from * S + to] += 1.0;
            for (int i = 0; i < N; ++i)
                if (occupation[i]) occupations_in_time[i] += hop_time;
        }
        time += hop_time;
        if (hop_log) { hop_log[2 * hop] = from; hop_log[2 * hop + 1] = to; }
        if (hop_times) hop_times[hop] = hop_time;
    }
    *time_out = time;
    free(se);
    free(cum);
    return 0;
}

static inline uint64_t splitmix64(uint64_t x);

/* A replay stream on which every hop's event uniform lies at least
 * min_margin (as a fraction of the total rate) from the cumulative
 * boundaries of the pair it selects: the numba loop above is run on uniforms
 * from SplitMix64 (seed), and an event uniform closer than min_margin to a
 * boundary is replaced by the generator's next value (at most 100000 tries).
 * Any hop loop whose cumulative rates are within min_margin of the FP64
 * ones must then follow the FP64 hop sequence on this stream exactly.
 * occupation (N) is the start state and is not modified; site_energies (S)
 * carries the electrode energies at [N, S).  uniforms_out gets
 * 2*hops values in (0,1); *redraws the number of replaced uniforms.
 * Returns 0, -1 on bad arguments, -2 on allocation failure, -3 when no
 * clear uniform was found for some hop. */
int oracle_clear_stream(int N, int P, double nu, double kT, double I_0, double R,
                        const uint8_t *occupation_in, const double *distances,
                        const double *E_constant, const double *site_energies_in,
                        const double *transitions_constant, int64_t hops, uint64_t seed,
                        double min_margin, double *uniforms_out, int64_t *redraws)
{
    const int S = N + P;
    if (N < 0 || P < 0 || S <= 0 || hops < 0 || !uniforms_out) return -1;
    double *se = (double *)malloc(sizeof(double) * (size_t)S);
    double *cum = (double *)malloc(sizeof(double) * (size_t)S * (size_t)S);
    uint8_t *occ = (uint8_t *)malloc((size_t)(N > 0 ? N : 1));
    if (!se || !cum || !occ) { free(se); free(cum); free(occ); return -2; }
    if (N > 0) memcpy(occ, occupation_in, (size_t)N);
    memcpy(se, site_energies_in, sizeof(double) * (size_t)S);   /* electrode energies at [N, S) */
    uint64_t ctr = 0;
    int64_t nre = 0;
    int rc = 0;
    const uint64_t golden = 0x9E3779B97F4A7C15ULL;
    for (int64_t hop = 0; hop < hops && rc == 0; ++hop) {
        const double total = numba_state_rates(N, P, nu, kT, I_0, R, occ, distances, E_constant,
                                               transitions_constant, se, cum);
        const double u1 = ((double)(splitmix64(seed + (++ctr) * golden) >> 11) + 0.5) * 0x1.0p-53;
        double u2 = 0.0, mg = -1.0;
        size_t ev = 0;
        int tries = 0;
        for (; tries < 100000; ++tries) {
            u2 = ((double)(splitmix64(seed + (++ctr) * golden) >> 11) + 0.5) * 0x1.0p-53;
            ev = numba_select(cum, (size_t)S * S, total, u2, &mg);
            if (mg >= min_margin) break;
        }
        if (mg < min_margin) rc = -3;
        nre += tries;
        uniforms_out[2 * hop] = u1;
        uniforms_out[2 * hop + 1] = u2;
        const int from = (int)(ev / (size_t)S), to = (int)(ev % (size_t)S);
        if (from < N) occ[from] = 0;
        if (to < N) occ[to] = 1;
    }
    if (redraws) *redraws = nre;
    free(se);
    free(cum);
    free(occ);
    return rc;
}

/* ----------------------------------------------------------------------- */
/* Go-path restatement (FP32, incremental energies, no memo)                 */
/* ----------------------------------------------------------------------- */

static inline uint64_t splitmix64(uint64_t x)
{
    uint64_t z = x;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

typedef struct { int from, to; float rate; } go_trans;

/* One chain.  Tables are FP64 S*S inputs converted to FP32 like
 * deFlattenFloatTo32 (simulationWrapper.go:37-48).  occupation is the start
 * state (wrapperSimulate passes it empty); it is updated in place.
 * electrode_occupation (P doubles) is zeroed then accumulated.  traffic
 * (S*S) and average_occupation (N) are accumulated when record != 0.
 * Returns the simulated time; *n_exp receives the number of rate
 * evaluations that took the exponential branch or not (allowed pairs). */
double oracle_go_simulate(int N, int P, double nu_d, double kT_d, double I0_d, double R_d,
                          uint8_t *occupation, const double *distances,
                          const double *E_constant, const double *site_energies_in,
                          const double *transitions_constant, double *electrode_occupation,
                          int64_t hops, int record, double *traffic, double *average_occupation,
                          uint64_t seed, int64_t *n_allowed)
{
    const int S = N + P;
    const float nu = (float)nu_d, kT = (float)kT_d, I0 = (float)I0_d, R = (float)R_d;
    float *d32 = (float *)malloc(sizeof(float) * (size_t)S * S);
    float *tc32 = (float *)malloc(sizeof(float) * (size_t)S * S);
    float *se = (float *)malloc(sizeof(float) * (size_t)S);
    go_trans *tl = (go_trans *)malloc(sizeof(go_trans) * (size_t)S * S);
    float *plist = (float *)malloc(sizeof(float) * (size_t)S * S);
    if (!d32 || !tc32 || !se || !tl || !plist) {
        free(d32); free(tc32); free(se); free(tl); free(plist);
        return -1.0;
    }
    for (size_t k = 0; k < (size_t)S * S; ++k) {
        d32[k] = (float)distances[k];
        tc32[k] = (float)transitions_constant[k];
    }
    for (int i = 0; i < S; ++i) se[i] = (float)site_energies_in[i];
    /* transition list: tc > 0 * max(tc) (cut = 0), simulation.go:199-215 */
    int nt = 0;
    for (int i = 0; i < S; ++i)
        for (int j = 0; j < S; ++j)
            if (tc32[(size_t)i * S + j] > 0.0f) { tl[nt].from = i; tl[nt].to = j; tl[nt].rate = 0; ++nt; }
    /* initial energies, simulation.go:226-234 */
    for (int i = 0; i < N; ++i) {
        float acc = 0.0f;
        for (int j = 0; j < N; ++j)
            if (j != i && !occupation[j]) acc += 1.0f / d32[(size_t)i * S + j];
        se[i] = (float)E_constant[i] - I0 * R * acc;
    }
    for (int e = 0; e < P; ++e) electrode_occupation[e] = 0.0;
    double time = 0.0;
    int64_t allowed = 0;
    for (int64_t hop = 0; hop < hops; ++hop) {
        /* calcTransitionList, simulation.go:58-80 */
        for (int k = 0; k < nt; ++k) {
            int i = tl[k].from, j = tl[k].to;
            int ok;
            if (i == j) ok = 0;
            else if (i >= N && j >= N) ok = 0;
            else if (i >= N && occupation[j]) ok = 0;
            else if (j >= N && !occupation[i]) ok = 0;
            else if (i < N && j < N && (!occupation[i] || occupation[j])) ok = 0;
            else ok = 1;
            if (!ok) { tl[k].rate = 0.0f; continue; }
            ++allowed;
            float dE;
            if (i < N && j < N) dE = se[j] - se[i] - I0 * R / d32[(size_t)i * S + j];
            else dE = se[j] - se[i];
            float r = (dE > 0) ? nu * (float)exp((double)(-dE / kT)) : nu;
            tl[k].rate = r * tc32[(size_t)i * S + j];
        }
        for (int k = 0; k < nt; ++k) plist[k] = (k == 0) ? tl[0].rate : plist[k - 1] + tl[k].rate;
        const uint64_t base = seed * 0x2545F4914F6CDD1DULL + (uint64_t)hop * 2ULL;
        double u1 = ((double)(splitmix64(base + 1) >> 11) + 0.5) * 0x1.0p-53;
        float u2 = (float)((double)(splitmix64(base + 2) >> 40) * 0x1.0p-24);
        const double time_step = -log(u1) / (double)plist[nt - 1];
        time += time_step;
        /* getRandomEvent, simulation.go:163-188 */
        const float eventRand = u2 * plist[nt - 1];
        int e_step = nt / 2, i = e_step, event = 0;
        for (;;) {
            if (e_step >= 2) e_step /= 2;
            if (plist[i] < eventRand) {
                i += e_step;
                if (i >= nt) i = nt - 1;
            } else if (i > 0 && plist[i - 1] >= eventRand) {
                i -= e_step;
                if (i < 0) i = 0;
            } else {
                event = i;
                break;
            }
        }
        const int from = tl[event].from, to = tl[event].to;
        if (record) {
            traffic[(size_t)from * S + to] += 1.0;
            traffic[(size_t)to * S + from] -= 1.0;
            for (int a = 0; a < N; ++a)
                if (occupation[a]) average_occupation[a] += time_step;
        }
        /* makeJump, simulation.go:107-130 */
        if (from < N) {
            occupation[from] = 0;
            for (int j = 0; j < N; ++j)
                if (j != from) se[j] -= I0 * R * (1.0f / d32[(size_t)j * S + from]);
        } else {
            electrode_occupation[from - N] -= 1.0;
        }
        if (to < N) {
            occupation[to] = 1;
            for (int j = 0; j < N; ++j)
                if (j != to) se[j] += I0 * R * (1.0f / d32[(size_t)j * S + to]);
        } else {
            electrode_occupation[to - N] += 1.0;
        }
    }
    if (n_allowed) *n_allowed = allowed;
    free(d32); free(tc32); free(se); free(tl); free(plist);
    return time;
}

/* A range of chains sharing one geometry, each with its own E_constant row,
 * electrode energies and seed: the CPU baseline of the batched engine.
 * Threads are created by the caller (one call per thread). */
int oracle_go_chains(int N, int P, double nu, double kT, double I0, double R,
                     const uint8_t *occupation0, const double *distances,
                     const double *E_constant_rows, const double *site_energies_rows,
                     const double *transitions_constant, int64_t hops,
                     int64_t first, int64_t count, uint64_t seed,
                     double *times_out, double *eo_out, int64_t *n_allowed_out)
{
    const int S = N + P;
    uint8_t *occ = (uint8_t *)malloc((size_t)(N > 0 ? N : 1));
    if (!occ) return -2;
    for (int64_t c = first; c < first + count; ++c) {
        memcpy(occ, occupation0 + (size_t)c * N, (size_t)N);
        int64_t na = 0;
        times_out[c] = oracle_go_simulate(N, P, nu, kT, I0, R, occ, distances,
                                          E_constant_rows + (size_t)c * N,
                                          site_energies_rows + (size_t)c * S,
                                          transitions_constant, eo_out + (size_t)c * P,
                                          hops, 0, NULL, NULL, seed + (uint64_t)c, &na);
        if (n_allowed_out) n_allowed_out[c] = na;
    }
    free(occ);
    return 0;
}


/* ----------------------------------------------------------------------- */
/* Go mean-field restatement                                                 */
/* ----------------------------------------------------------------------- */

/* probSimulate, goSimulation/probabilitySimulation.go:53-157.  occupation
 * (N, in/out, probabilities), electrode_occupation (P, out: integrated net
 * flow into each electrode), site_energies (N, out), traffic (S*S) and
 * average_occupation (N) accumulated when record != 0.  Returns the
 * simulated time, or -1 on bad arguments / allocation failure. */
double oracle_prob_simulate(int N, int P, double nu, double kT, double I_0, double R,
                            double *occupation, const double *distances, const double *E_constant,
                            const double *tc, double *electrode_occupation, double *site_energies,
                            int hops, int record, double *traffic, double *average_occupation)
{
    if (N < 0 || P < 0 || N + P < 1 || hops < 0) return -1.0;
    const int S = N + P;
    double *t = (double *)malloc(sizeof(double) * (size_t)S * S);
    double *difference = (double *)malloc(sizeof(double) * (size_t)(N > 0 ? N : 1));
    if (!t || !difference) { free(t); free(difference); return -1.0; }
    for (int e = 0; e < P; ++e) electrode_occupation[e] = 0.0;
    double time = 0.0;
    for (int hop = 0; hop < hops; ++hop) {
        /* site energies from the occupation probabilities (:85-94); the
         * electrode entries site_energies[N..S) are the voltages */
        for (int i = 0; i < N; ++i) {
            difference[i] = 0.0;
            double acc = 0.0;
            for (int j = 0; j < N; ++j)
                if (j != i) acc += (1.0 - occupation[j]) / distances[i * S + j];
            site_energies[i] = E_constant[i] - I_0 * R * acc;
        }
        /* expected rates, their total and the net flow per site, row-major
         * (calcProbTransitions :7-35, probTransitionPossible :37-49) */
        double tot = 0.0;
        for (int i = 0; i < S; ++i) {
            for (int j = 0; j < S; ++j) {
                double base;
                if (i >= N && j >= N) base = 0.0;
                else if (i >= N) base = 1.0 - occupation[j];
                else if (j >= N) base = occupation[i];
                else base = (1.0 - occupation[j]) * occupation[i];
                double dE;
                if (i < N && j < N) dE = site_energies[j] - site_energies[i] - I_0 * R / distances[i * S + j];
                else dE = site_energies[j] - site_energies[i];
                double r = dE > 0 ? base * nu * exp(-dE / kT) : base * nu;
                r *= tc[i * S + j];
                t[i * S + j] = r;
                tot += r;
                if (i < N) difference[i] -= r;
                if (j < N) difference[j] += r;
            }
        }
        /* largest step that keeps every probability in [0, 1] (:95-110) */
        double max_change = 1.0;
        for (int i = 0; i < N; ++i) {
            const double nv = occupation[i] + difference[i] / tot;
            if (nv < 0) {
                const double req = occupation[i] / -(difference[i] / tot);
                if (req < max_change) max_change = req;
            }
            if (nv > 1) {
                const double req = (1.0 - occupation[i]) / (difference[i] / tot);
                if (req < max_change) max_change = req;
            }
        }
        const double time_step = 0.98 * max_change / tot;
        time += time_step;
        if (record)
            for (int i = 0; i < N; ++i) average_occupation[i] += occupation[i] * time_step;
        /* move the expected charge (:118-142) */
        for (int i = 0; i < S; ++i) {
            for (int j = 0; j < S; ++j) {
                if (i >= N && j >= N) break;
                const double rate = t[i * S + j] * max_change / tot;
                if (i < N) occupation[i] -= rate; else electrode_occupation[i - N] -= rate;
                if (j < N) occupation[j] += rate; else electrode_occupation[j - N] += rate;
                if (record) {
                    traffic[i * S + j] += rate;
                    traffic[j * S + i] -= rate;
                }
            }
        }
        /* clamp (:143-152) */
        for (int i = 0; i < N; ++i) {
            if (occupation[i] < 0) occupation[i] = 0;
            if (occupation[i] > 1) occupation[i] = 1;
        }
    }
    free(t); free(difference);
    return time;
}
