/*
 * kmc_dn_gb300.h -- C ABI of the GB300 (sm_103a) kinetic Monte Carlo engine
 * for dopant networks.
 *
 * This is the drop-in boundary for the hop loop of MUTUEL/kmc_dn.  The
 * reference reaches its native loop through ctypes on a Go c-shared library
 * (goSimulation/pythonBind.py:49-92, goSimulation/parrallelSimulationBind.py:
 * 50-66) whose exports take GoSlice {data, len, cap} views of FP64 host
 * arrays (goSimulation/simulationWrapper.go:83-315).  The entry points below
 * take plain pointers and sizes, return a status code, and never abort the
 * host process.  Each declaration names the reference interface it replaces.
 *
 * Conventions
 *   - S = N + P sites, acceptors first, then electrodes (the reference's
 *     site order, kmc_dopant_networks.py:657-695).  Pair tables are S*S,
 *     row-major (from, to).
 *   - "device" pointers are CUDA device (or managed) memory; "host"
 *     pointers are ordinary host memory.
 *   - stream: a cudaStream_t passed as void* (NULL = the legacy default
 *     stream).  Device-pointer entry points are asynchronous on that stream;
 *     host-pointer entry points synchronise before returning.
 *   - Return value: KMC_OK (0) or a negative KMC_ERR_* code; the message of
 *     the last error on the calling thread is read with kmc_last_error().
 *     Per-chain problems (no allowed transition, non-finite total rate)
 *     are reported per chain in a status array and do not fail the call.
 */
#ifndef KMC_DN_GB300_H
#define KMC_DN_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KMC_OK 0
#define KMC_ERR_INVALID (-1)    /* bad sizes, pointers or options            */
#define KMC_ERR_CUDA (-2)       /* a CUDA runtime call failed                */
#define KMC_ERR_OOM (-3)        /* device or host allocation failed          */
#define KMC_ERR_TIMEOUT (-4)    /* hop or wall-clock budget exhausted        */
#define KMC_ERR_NONFINITE (-5)  /* total rate zero, negative or non-finite   */
#define KMC_ERR_CANCELLED (-6)  /* stopped through the cancel word           */

/* Version of this ABI (major*10000 + minor*100 + patch). */
int kmc_version(void);

/* Copy the last error message of the calling thread into buf (always NUL
 * terminated); returns the last status code.  No reference counterpart: the
 * Go library has no error channel (goSimulation/pythonBind.py:81). */
int kmc_last_error(char *buf, size_t len);

/* ------------------------------------------------------------------------ */
/* Plain single-chain FP64 hop loop                                          */
/* ------------------------------------------------------------------------ */

/* Workspace bytes kmc_simulate_f64 needs for S sites. */
size_t kmc_simulate_f64_workspace_size(int32_t n_sites);

/*
 * One chain, FP64 throughout, with the semantics of the reference's numba
 * loop _simulate_discrete_record (kmc_dopant_networks.py:33-135), which
 * kmc_dn.python_simulation / makeSimulation call (:513-619):
 *   - starts from `occupation` and leaves the final state in it;
 *   - electrode_occupation is accumulated (+1 = a hole into the electrode);
 *   - each hop draws two uniforms, clock first: dt = -log(1-u1) / total,
 *     then the first row-major pair k with cum_k/total >= u2 (:100-110);
 *   - record != 0: traffic[from*S+to] += 1 and occupations_in_time[i] +=
 *     dt for every acceptor occupied AFTER the hop (:126-130).
 * uniforms: NULL, or 2*hops replay values in (0,1) (device).  When NULL the
 * uniforms come from Philox4x32-10 keyed by seed.
 * All arrays are device pointers; hop_log (2*hops int32) may be NULL;
 * time_out and status_out are single device values.  workspace must hold
 * kmc_simulate_f64_workspace_size(S) bytes.
 */
int kmc_simulate_f64(int32_t n_acceptors, int32_t n_electrodes, double nu, double kT,
                     double I_0, double R, uint8_t *occupation, const double *distances,
                     const double *E_constant, const double *site_energies,
                     const double *transitions_constant, int64_t *electrode_occupation,
                     int64_t hops, int32_t record, double *traffic,
                     double *occupations_in_time, const double *uniforms, uint64_t seed,
                     int32_t *hop_log, double *time_out, int32_t *status_out,
                     void *workspace, size_t workspace_bytes, void *stream);

/*
 * kmc_simulate_f64 that also accumulates, into flux_time (P device doubles,
 * at most 64 electrodes), the time integral of each electrode's expected
 * net hole inflow: in every state, column N+e minus row N+e of the FP64 rate
 * matrix, times the hop's time.  electrode_occupation minus flux_time is a
 * zero-mean martingale, so flux_time / time is a low-variance companion
 * estimate of the current, used to compare precisions.  The hop sequence is
 * that of kmc_simulate_f64.  No reference counterpart (measurement support
 * for the loop kmc_dopant_networks.py:33-135).
 */
int kmc_simulate_f64_flux(int32_t n_acceptors, int32_t n_electrodes, double nu, double kT,
                          double I_0, double R, uint8_t *occupation, const double *distances,
                          const double *E_constant, const double *site_energies,
                          const double *transitions_constant, int64_t *electrode_occupation,
                          int64_t hops, int32_t record, double *traffic,
                          double *occupations_in_time, const double *uniforms, uint64_t seed,
                          int32_t *hop_log, double *time_out, int32_t *status_out,
                          void *workspace, size_t workspace_bytes, void *stream,
                          double *flux_time);

/*
 * Many independent plain FP64 chains in one launch (one thread block per
 * chain), for FP64 statistics beside the batched FP32 engine: each chain is
 * kmc_simulate_f64 in Philox mode (its own seed, no replay, no hop log).
 * Every pointer is device memory; per-chain segments are given by offsets:
 *   pair_off[c]   S*S block of distances / transitions_constant (shareable),
 *   site_off[c]   N entries of E_constant, occupation (in/out) and, with
 *                 record, occupations_in_time (accumulated),
 *   se_off[c]     S entries of site_energies (electrode energies at [N, S)),
 *   el_off[c]     P entries of electrode_occupation (accumulated) and of
 *                 flux_time (optional, accumulated; at most 64 electrodes),
 *   traffic_off[c] S*S block of traffic (record only, accumulated).
 * time_out[c] and status_out[c] (KMC_OK, KMC_ERR_NONFINITE, or
 * KMC_ERR_INVALID for a chain whose sizes exceed max_sites) are written.
 * The workspace holds kmc_simulate_f64_batch_workspace_size(n_chains,
 * max_sites) bytes.  Replaces running the reference's numba loop once per
 * chain (kmc_dopant_networks.py:33-135).
 */
typedef struct kmc_f64_batch {
    int32_t n_chains;
    int32_t max_sites;              /* >= N + P of every chain                 */
    int32_t record;                 /* 0 / 1 (numba convention)                */
    const int32_t *N, *P;
    const double *nu, *kT, *I_0, *R;
    const int64_t *pair_off;
    const double *distances, *transitions_constant;
    const int64_t *site_off;
    const double *E_constant;
    const int64_t *se_off;
    const double *site_energies;
    uint8_t *occupation;
    const int64_t *el_off;
    int64_t *electrode_occupation;
    const int64_t *hops;
    const uint64_t *seeds;
    const int64_t *traffic_off;
    double *traffic;
    double *occupations_in_time;
    double *time_out;
    int32_t *status_out;
    double *flux_time;              /* optional                                */
    double *workspace;
    size_t workspace_bytes;
} kmc_f64_batch;

size_t kmc_simulate_f64_batch_workspace_size(int32_t n_chains, int32_t max_sites);
int kmc_simulate_f64_batch(const kmc_f64_batch *batch, void *stream);

/*
 * kmc_simulate_f64 without a workspace argument, for callers that cannot
 * allocate device memory at the point of the call: a host application that
 * owns the device through its own memory pool and passes this library only
 * the buffers it placed, or a latency-bound loop where cudaMalloc/cudaFree
 * (which can synchronise the device) are not acceptable.  No counterpart in
 * the reference (its Go library allocates freely on the host).
 *   - The workspace is a fixed array inside this library: networks of at
 *     most 128 sites (N + P); larger ones return KMC_ERR_INVALID with a
 *     message.  The array (384 KiB) stays resident on every device that
 *     loads the library's device code until the process exits.
 *   - Under CUDA's default lazy module loading the device code (and with it
 *     the array) is loaded into a context at its first use there, which
 *     for a caller of this entry alone is its first call on a device: that
 *     first call does take device memory.  Make one warm-up call on each
 *     device (or load with CUDA_MODULE_LOADING=EAGER) before your own pool
 *     takes the device, and before any stream capture on it.  Later calls
 *     allocate nothing.
 *   - Every call looks the array's device address up in the current
 *     context (cudaGetSymbolAddress), so the entry stays valid after a
 *     cudaDeviceReset and in a non-primary context.
 *   - All calls share the one array: calls whose kernels overlap on the
 *     device (different streams, or host threads) race and corrupt each
 *     other's results.  Serialise them on one stream.
 *   - Everything else (arguments, semantics, asynchrony) is that of
 *     kmc_simulate_f64.  The call allocates nothing.
 */
int kmc_simulate_f64_static(int32_t n_acceptors, int32_t n_electrodes, double nu, double kT,
                            double I_0, double R, uint8_t *occupation, const double *distances,
                            const double *E_constant, const double *site_energies,
                            const double *transitions_constant, int64_t *electrode_occupation,
                            int64_t hops, int32_t record, double *traffic,
                            double *occupations_in_time, const double *uniforms, uint64_t seed,
                            int32_t *hop_log, double *time_out, int32_t *status_out,
                            void *stream);

/* ------------------------------------------------------------------------ */
/* Batched FP32 engine                                                       */
/* ------------------------------------------------------------------------ */

/* Record conventions. */
#define KMC_RECORD_NONE 0
#define KMC_RECORD_NUMBA 1   /* traffic[f,t] += 1; occupancy credited after the hop
                                (kmc_dopant_networks.py:126-130) */
#define KMC_RECORD_GO 2      /* traffic[f,t] += 1, traffic[t,f] -= 1; occupancy
                                credited before the hop (simulation.go:309-317) */

/* Where the engine takes L = log2(nu*tc_ij) and B = I_0 R / d_ij from. */
#define KMC_PAIRS_TABLE 0      /* per-geometry pair table (tab_LB): any tables */
#define KMC_PAIRS_POSITIONS 1  /* site coordinates (tab_pos): tc = nu*exp(-2d/ab),
                                  the reference's calc_transitions_constant
                                  (kmc_dopant_networks.py:824-830); only valid
                                  when the tables are those of the positions */

/*
 * Launch description of the batched engine.  Every pointer is device
 * memory.  A "table" is one geometry instance: S*S interleaved float pairs
 * (L, B) with L = log2(nu * transitions_constant[i][j]) and B = I_0*R /
 * distances[i][j] for acceptor pairs, 0 otherwise (built from the FP64
 * tables by kmc_build_tables).  Chains name a table; many chains may share
 * one.  Per-site pools (N entries per chain), per-electrode pools (P
 * entries per chain) and per-pair pools (S*S entries per chain) are indexed
 * by the chain's offsets.
 *
 * The work list assigns chains to thread groups.  For G <= 32 lanes per
 * chain, item w is 32/G chain ids work[w*(32/G) + s] (-1 = empty slot) run
 * by one warp; for G in {64, 128, 256, 512}, item w is one chain id run by
 * one block of G threads.  Chains in one item should have similar size and
 * hop budget.
 *
 * Each launch advances every listed chain by min(hops_total - hops_done,
 * max_hops_per_launch) hops (max_hops_per_launch a multiple of reanchor),
 * accumulating time, electrode_occupation and the record pools, and
 * writing back occupation and hops_done, so a run can be split into
 * launches (serving, checkpoint/resume) with results independent of the
 * split.
 */
typedef struct kmc_batch {
    /* tables */
    int32_t n_tables;
    int32_t max_sites;              /* >= S of every chain in the launch       */
    const int32_t *tab_N;           /* [n_tables] acceptors                    */
    const int32_t *tab_P;           /* [n_tables] electrodes (<= 64)           */
    const int64_t *tab_off;         /* [n_tables] offset in floats into tab_LB */
    const float *tab_LB;            /* pair tables, 2*S*S floats each          */
    /* chains */
    int32_t n_chains;
    int32_t lanes_per_chain;        /* G in {4, 8, 16, 32, 64, 128, 256, 512}  */
    const int32_t *chain_tab;       /* [n_chains]                              */
    const float *chain_kT;          /* [n_chains]                              */
    const int64_t *chain_site_off;  /* [n_chains] offset into per-site pools   */
    const int64_t *chain_el_off;    /* [n_chains] offset into electrode pools  */
    const int64_t *chain_pair_off;  /* [n_chains] offset into traffic pool     */
    const float *E_constant;        /* site pool: constant site energies       */
    const float *el_energy;         /* electrode pool: electrode energies      */
    uint8_t *occupation;            /* site pool, in/out                       */
    int64_t *electrode_occupation;  /* electrode pool, accumulated             */
    double *time;                   /* [n_chains] accumulated                  */
    int64_t *hops_done;             /* [n_chains] in/out                       */
    const int64_t *hops_total;      /* [n_chains]                              */
    const uint64_t *stream;         /* [n_chains] RNG stream ids               */
    int32_t *status;                /* [n_chains] out: KMC_OK or KMC_ERR_*     */
    unsigned long long *n_pairs;    /* [n_chains] accumulated allowed pairs    */
    double *occ_time;               /* site pool: time-weighted occupancy      */
    double *occ_since;              /* site pool: scratch for occ_time         */
    int32_t *traffic;               /* pair pool                               */
    /* work list */
    const int32_t *work;
    int32_t n_work;
    int32_t record;                 /* KMC_RECORD_*                            */
    int32_t reanchor;               /* hops between FP32 energy re-anchors     */
    int32_t warps_per_block;        /* 1..8                                    */
    int64_t max_hops_per_launch;
    uint64_t seed;
    const double *replay;           /* optional 2 uniforms per hop per chain   */
    const int64_t *replay_off;      /* [n_chains] offset into replay           */
    const volatile int32_t *cancel; /* optional host-mapped cancel word        */
    /* pair rates from coordinates instead of tables (KMC_PAIRS_POSITIONS) */
    int32_t pair_mode;              /* KMC_PAIRS_TABLE or KMC_PAIRS_POSITIONS  */
    const float *tab_pos;           /* sites' (x, y, z, 0), 4 floats per site  */
    const int64_t *tab_pos_off;     /* [n_tables] offset in floats into tab_pos*/
    const float *tab_coef;          /* [n_tables*4]: -2*log2(e)/ab,
                                       log2(nu*nu), I_0*R, 0                   */
    /* wall-clock budget of one launch per chain, checked with the cancel word
     * every 1024 hops (not before the first 1024 of a launch); a chain that
     * overruns stops with KMC_ERR_TIMEOUT at a multiple of 1024 hops, its
     * state consistent, and a later launch resumes it as if uninterrupted.
     * 0: none */
    int64_t time_budget_ns;
    /* optional per-hop log (replay tests, rate-level accuracy checks): the
     * chain's absolute hop k (k < hops_total[c]) writes {from, to} to
     * hop_log[2*(hop_log_off[c] + k)] and, when hop_rates is set, {total
     * rate, rate of the chosen pair} as the engine computed them (FP32) to
     * hop_rates[2*(hop_log_off[c] + k)].  NULL: no log */
    int32_t *hop_log;
    float *hop_rates;
    const int64_t *hop_log_off;     /* [n_chains] offset in hops               */
    /* debug builds only (-DKMC_DEBUG_CHECKS): per chain, hops whose event an
     * FP64 scan and compare over the same FP32 per-thread sums would place
     * on another pair than the engine's exact integer compare; NULL: off */
    unsigned long long *select_mismatch;
    /* optional, per chain: the largest difference (in units of kT) between
     * the FP32 energies the O(N) incremental updates carried and the same
     * energies recomputed from scratch, taken at every re-anchor (every
     * `reanchor` hops): the drift the periodic re-anchor removes.  Kept as
     * a running maximum over launches.  NULL: not measured */
    float *energy_drift;
    /* optional: a device counter, zero at launch, that makes the launch
     * persistent -- as many blocks as stay resident, each warp (warp slices)
     * or block (block groups) claiming the next work item with an atomic
     * add when its chains are done, instead of one item per warp for the
     * whole launch.  Results do not depend on it.  NULL: static launch */
    int32_t *work_counter;
    /* optional, electrode pool (P doubles per chain), accumulated: the time
     * integral of each electrode's expected net inflow J_e = sum over holes
     * of rate(i -> e) - sum over empty acceptors of rate(e -> j), taken in
     * every state for the time spent in it.  electrode_occupation minus this
     * is a zero-mean martingale, so it is a low-variance companion estimate
     * of the current (accuracy checks).  NULL: not computed */
    double *flux_time;
    /* persistent launches only: at most this many blocks (0: as many as
     * stay resident), so that launches of several size bins running side by
     * side can share the device in proportion to their work */
    int32_t max_grid;
    /* > 0: every chain of the launch has this kT (the engine then stages a
     * single pair table with the temperature folded in; a chain whose kT
     * differs stops with KMC_ERR_INVALID).  0: per-chain kT as given */
    float uniform_kT;
} kmc_batch;

/*
 * Build one FP32 pair table (2*S*S floats at tab_LB) from FP64 device
 * tables: L = log2(nu*tc), B = I_0*R/d for acceptor pairs.  Restates the
 * constant part of the rate (calc_transitions_constant,
 * kmc_dopant_networks.py:824-830) and the Coulomb term of dE
 * (:72-75, simulation.go:67-68) in the form the engine consumes.
 */
int kmc_build_table(int32_t n_acceptors, int32_t n_electrodes, double nu, double I_0, double R,
                    const double *distances, const double *transitions_constant,
                    float *tab_LB, void *stream);

/*
 * Constant site energies of many chains on one geometry from the Laplace
 * basis fields sampled at the acceptors (the linear superposition that
 * replaces a FEniCS solve per voltage vector, kmc_dopant_networks.py:
 * 798-821 + 865-899):
 *   E_constant[c][i] = sum_e V[c][e]*basis[e][i] + mu*basis[n_el][i] + comp[i]
 *   el_energy[c][e]  = V[c][e]
 * basis: (n_el+1) x N FP64, V: n_chains x n_el FP64, comp: N FP64.
 * Outputs: E_constant FP32 (n_chains x N, row stride N), el_energy FP32.
 */
int kmc_site_energies(int32_t n_chains, int32_t n_acceptors, int32_t n_electrodes,
                      const double *basis, const double *voltages, double mu,
                      const double *comp, float *E_constant, float *el_energy, void *stream);

/*
 * Run one launch of the batched engine (device pointers, asynchronous).
 * Replaces the goroutine-per-chain parallelSimulations
 * (goSimulation/simulationWrapper.go:275-315) and the per-chain Go
 * simulate loop (simulation.go:194-325).
 */
int kmc_run_batch(const kmc_batch *batch, void *stream);

/* Lanes-per-chain choices compiled into the engine: bit k set = G of 2^k. */
int kmc_engine_lane_options(void);

/* Per-phase SM-clock cycles of the FP32 engine's hop loop, summed over the
 * chains of every launch since the last reset (thread 0 of each group):
 * cycles[0..7] = loop checks, pair walk, uniforms, group scan and target,
 * event search, clock, energy update and list rebuild, hop bookkeeping;
 * cycles[8] = hops.  reset != 0 zeroes the counters after reading.  Only a
 * library built with -DKMC_SECTION_CLOCKS (kmc_dn_gb300/build.py
 * --section-clocks) counts; the release library returns KMC_ERR_INVALID.
 * No reference counterpart (measurement support). */
int kmc_section_clocks(uint64_t *cycles, int32_t reset);

/* Measure the device's ex2 (SFU) throughput in ex2 results per second: the
 * roofline of the rate evaluation.  Synchronous, on the current device.  No
 * reference counterpart (measurement support). */
int kmc_measure_ex2_rate(double *ex2_per_second);

/* Load every kernel of the library on the current device now.  CUDA loads
 * a kernel's code lazily at its first launch, and that load waits for the
 * kernels already running: a size class launched for the first time beside
 * running ones (the uneven batch's bins on their own streams, a serving
 * loop's new class) would otherwise start only when they end.  Idempotent;
 * call once per device before concurrent launches.  No reference
 * counterpart (the Go library runs on the host). */
int kmc_preload_kernels(void);

/*
 * Host-buffer batch run: chains on shared geometries, FP64 host inputs,
 * copies in and out inside the call (synchronous).  This is the
 * reference-facing batched call with host buffers, the counterpart of
 * parallelSimulations (goSimulation/simulationWrapper.go:275-315) fed by
 * parrallelSimulation.runSimulation (goSimulation/parrallelSimulationBind.py:
 * 50-66), with per-geometry instead of per-chain tables.
 *   geometries g: N[g], P[g], nu[g], I_0[g], R[g], distances/tc at
 *     geom_pair_off[g] (S*S FP64 each) in `distances`/`transitions_constant`.
 *   chains c: chain_geom[c], kT[c], E_constant (N FP64 at site offset),
 *     site_energies (S FP64, electrode energies at [N..S)), occupation
 *     (N bytes, in/out), hops[c], seed.
 *   outputs: time[c], electrode_occupation (P int64 per chain, overwritten),
 *     status[c].
 * lanes_per_chain 0 = choose automatically.
 */
int kmc_run_batch_host(int32_t n_geoms, const int32_t *geom_N, const int32_t *geom_P,
                       const double *geom_nu, const double *geom_I0, const double *geom_R,
                       const int64_t *geom_pair_off, const double *distances,
                       const double *transitions_constant, int32_t n_chains,
                       const int32_t *chain_geom, const double *chain_kT,
                       const double *E_constant, const double *site_energies,
                       uint8_t *occupation, const int64_t *hops, uint64_t seed,
                       int32_t lanes_per_chain, double *time_out,
                       int64_t *electrode_occupation, int32_t *status);

/* ------------------------------------------------------------------------ */
/* Resident engine handle: chain state stays on the device between runs     */
/* (the resident / serving mode; the reference has no counterpart -- its Go  */
/* calls, simulationWrapper.go:83-315, rebuild every state per call)        */
/* ------------------------------------------------------------------------ */

typedef struct kmc_engine kmc_engine;

/* Upload the geometries and chains (arguments as kmc_run_batch_host, host
 * buffers; record = KMC_RECORD_*) and keep them resident.  stream NULL: the
 * engine creates its own.  Nothing runs yet. */
int kmc_engine_create(kmc_engine **engine, int32_t n_geoms, const int32_t *geom_N, const int32_t *geom_P,
                      const double *geom_nu, const double *geom_I0, const double *geom_R,
                      const int64_t *geom_pair_off, const double *distances,
                      const double *transitions_constant, int32_t n_chains, const int32_t *chain_geom,
                      const double *chain_kT, const double *E_constant, const double *site_energies,
                      const uint8_t *occupation, const int64_t *hops, uint64_t seed,
                      int32_t lanes_per_chain, int32_t record, void *stream);
/* Advance every chain by up to max_hops more hops (rounded up to 1024; <= 0:
 * to its budget), asynchronously.  A run split into several calls gives the
 * results of a single call. */
int kmc_engine_run(kmc_engine *engine, int64_t max_hops);
/* Copy the current results to host buffers (any may be NULL) and wait for
 * the engine: time[n_chains], electrode_occupation[sum P], occupation
 * [sum N], status[n_chains], hops_done[n_chains]; with record, traffic
 * (S*S per chain, chain order) and occupations_in_time (N per chain). */
int kmc_engine_read(kmc_engine *engine, double *time_out, int64_t *electrode_occupation, uint8_t *occupation,
                    int32_t *status, int64_t *hops_done, double *traffic, double *occupations_in_time);
/* Free the engine's device memory (waits for its work). */
void kmc_engine_destroy(kmc_engine *engine);

/* ------------------------------------------------------------------------ */
/* Mean-field relaxation (replaces probSimulate / wrapperSimulateProbability, */
/* goSimulation/probabilitySimulation.go:53-157, simulationWrapper.go:224-235) */
/* ------------------------------------------------------------------------ */

#define KMC_MF_RATES_F64 0   /* exp() in FP64: the reference's arithmetic       */
#define KMC_MF_RATES_F32 1   /* ex2.approx.f32 rates, FP64 sums and state       */

/*
 * One network per chain; every pointer is a device pointer for kmc_mf_run and
 * a host pointer for kmc_mf_run_host.  Per-chain segments:
 *   pair_off[c]    S*S row-major block of distances / transitions_constant
 *                  (chains may share a block),
 *   site_off[c]    S-entry segment of E_constant (first N used),
 *                  site_energies (in: entries N..S-1 = electrode voltages;
 *                  out: entries 0..N-1 = the last iteration's energies),
 *                  occupation (first N: start probabilities in, final out)
 *                  and average_occupation (record: first N, time-weighted
 *                  probability sums, accumulated),
 *   el_off[c]      P entries of electrode_occupation (out: integrated net
 *                  expected charge into each electrode; the Go function
 *                  zeroes it first),
 *   traffic_off[c] S*S block of traffic (record: net expected flow i->j,
 *                  accumulated onto the caller's values).
 * time[c] receives the simulated time, status[c] KMC_OK or
 * KMC_ERR_NONFINITE (total rate zero or non-finite: the chain stops where
 * the Go loop would produce NaN), iterations_done[c] the iterations run.
 */
typedef struct kmc_mf_batch {
    int32_t n_chains;
    int32_t max_sites;              /* >= S of every chain, <= kmc_mf_max_sites */
    int32_t rates;                  /* KMC_MF_RATES_*                          */
    int32_t record;                 /* 0 / 1                                   */
    const int32_t *N;               /* [n_chains]                              */
    const int32_t *P;
    const double *nu, *kT, *I_0, *R;
    const int64_t *pair_off;
    const double *distances;
    const double *transitions_constant;
    const int64_t *site_off;
    const double *E_constant;
    double *site_energies;
    double *occupation;
    const int64_t *el_off;
    double *electrode_occupation;
    const int64_t *hops;            /* [n_chains] iterations (the Go "hops")   */
    const int64_t *traffic_off;     /* record only                             */
    double *traffic;
    double *average_occupation;
    double *time;                   /* [n_chains]                              */
    int32_t *status;                /* [n_chains] or NULL                      */
    int64_t *iterations_done;       /* [n_chains] or NULL                      */
} kmc_mf_batch;

/* A cancel word the host can set while kernels run (pinned, mapped host
 * memory): *host_word = 1 makes every chain of a launch that carries
 * device_word as kmc_batch.cancel stop at its next 1024-hop check with
 * KMC_ERR_CANCELLED, state consistent. */
int kmc_cancel_word_create(int32_t **host_word, int32_t **device_word);
void kmc_cancel_word_destroy(int32_t *host_word);

/* Largest S a chain may have for the given rate precision (its tables and
 * rates stay in one block's shared memory). */
int32_t kmc_mf_max_sites(int32_t rates);
/* Dynamic shared memory one block of kmc_mf_run uses. */
size_t kmc_mf_smem_bytes(int32_t max_sites, int32_t rates);
/* Device pointers, asynchronous on `stream`. */
int kmc_mf_run(const kmc_mf_batch *batch, void *stream);
/* Host pointers: copies in, runs, copies out, synchronises. */
int kmc_mf_run_host(const kmc_mf_batch *batch, void *stream);

/* ------------------------------------------------------------------------ */
/* Laplace basis fields on the device                                        */
/* ------------------------------------------------------------------------ */

/* Workspace bytes of kmc_laplace_basis for an nx x ny-cell mesh, n fields. */
size_t kmc_laplace_workspace_size(int32_t nx, int32_t ny, int32_t n_fields);

/*
 * Solve the Laplace problem of the reference's potential set-up (P1 elements
 * on a uniform right-triangle mesh with Dirichlet data on the whole boundary,
 * init_V/update_V, kmc_dopant_networks.py:706-822) for n_fields boundary
 * data sets at once.  grid (device, n_fields x (ny+1) x (nx+1), row = y
 * index) carries each field's boundary values on entry; its interior is
 * overwritten with the solution.  Exact direct solve by sine transforms.
 */
int kmc_laplace_basis(int32_t nx, int32_t ny, double hx, double hy, int32_t n_fields,
                      double *grid, void *workspace, size_t workspace_bytes, void *stream);

/* P1 interpolation of n_fields nodal grids at n_points (x, y) points
 * (device xy[2*n_points]); out[f*n_points + p].  The point evaluation of the
 * FEniCS function V(x, y) (kmc_dopant_networks.py:851-853). */
int kmc_p1_sample(int32_t nx, int32_t ny, double hx, double hy, int32_t n_fields,
                  const double *grid, int32_t n_points, const double *xy, double *out,
                  void *stream);

#ifdef __cplusplus
}
#endif

#endif /* KMC_DN_GB300_H */
