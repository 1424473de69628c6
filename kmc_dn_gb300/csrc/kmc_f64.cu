// kmc_f64.cu -- plain single-chain FP64 hop loop for sm_103a.
//
// One thread block runs one chain with the semantics of the reference's
// numba loop _simulate_discrete_record (kmc_dopant_networks.py:33-135), in
// FP64 and with the reference's operand order, so that fed the same uniform
// stream it makes the same hop sequence:
//
//   energies   E_i = Ec_i + (-I_0 R) * sum_{j != i} (1 - occ_j)/d_ij, summed in
//              ascending j (:59-66); 1/d_ij is tabulated once (the same
//              correctly rounded quotient the loop divides out each hop)
//   rates      dense S x S, row-major: tc_ij * (dE > 0 ? nu*exp(-dE/kT) : nu),
//              dE = E_j - E_i - (I_0 R)/d_ij for acceptor pairs (:69-87)
//   cumulative row-major running sum; each thread owns a contiguous chunk
//              and continues the running sum from the FP64 prefix of the
//              chunks before it (:91-97).  That prefix is a tree sum of the
//              chunk totals, not the reference's strictly left-to-right sum,
//              so cum_k and the total may differ in the last bit: the hop
//              sequence is the reference's except where u2 lies within a
//              few ulp of a boundary cum_k/total
//   clock      dt = -log(1 - u1) * (1/total) (:100)
//   event      first k with cum_k/total >= u2 (:103-110)
//   record     traffic[from,to] += 1, post-hop occupancy credit (:126-130)
//
// This is the baseline kernel the batched FP32 engine is measured against,
// and the kernel of the bit-exact replay check.
#include <cstdint>
#include <cuda_runtime.h>

#include "kmc_common.cuh"
#include "kmc_internal.h"

namespace kmc {
namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ bool possible(int i, int j, int N, const uint8_t *occ)
{
    if (i >= N && j >= N) return false;
    if (i >= N) return !occ[j];
    if (j >= N) return occ[i] != 0;
    if (i == j) return false;
    return occ[i] && !occ[j];
}

__device__ double block_exclusive_scan(double v, double *sh, double &total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const double o = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x += o;
    }
    if (lane == 31) sh[warp] = x;
    __syncthreads();
    if (warp == 0) {
        double w = lane < kThreads / 32 ? sh[lane] : 0.0;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const double o = __shfl_up_sync(0xffffffffu, w, d);
            if (lane >= d) w += o;
        }
        if (lane < kThreads / 32) sh[lane] = w;
    }
    __syncthreads();
    const double warp_base = warp > 0 ? sh[warp - 1] : 0.0;
    total = sh[kThreads / 32 - 1];
    __syncthreads();
    return warp_base + x - v;
}

// One chain run by the whole block (the body of both kernels below).
__device__ __forceinline__ void f64_chain(
    int N, int P, double nu, double kT, double I0, double R, uint8_t *occ_g, const double *d,
    const double *Ec, const double *se_in, const double *tc, int64_t *eo, int64_t hops,
    int record, double *traffic, double *oit, const double *uniforms, uint64_t seed,
    int32_t *hop_log, double *time_out, int32_t *status_out, double *ws, double *flux_time)
{
    extern __shared__ __align__(16) unsigned char sraw[];
    const int S = N + P;
    const int SS = S * S;
    double *se = reinterpret_cast<double *>(sraw);            // [S]
    double *red = se + S;                                     // [32] scan scratch
    uint8_t *occ = reinterpret_cast<uint8_t *>(red + 32);     // [S]
    __shared__ int ev_min;
    __shared__ double sh_total, sh_hop_time;
    __shared__ double sh_flux[64];   // expected net inflow of each electrode (flux_time only)

    double *invd = ws;                  // [N*N] 1/d_ij
    double *ird = ws + (size_t)N * N;   // [N*N] (I_0 R)/d_ij
    double *cum = ws + 2 * (size_t)N * N;   // [S*S] rates, then running sums

    const int tid = threadIdx.x;
    const bool kT_is_one = (kT == 1.0);
    const double IR = I0 * R;
    const double mIR = -I0 * R;
    for (int k = tid; k < N * N; k += kThreads) {
        const int i = k / N, j = k - (k / N) * N;
        const double dij = d[(size_t)i * S + j];
        invd[k] = (i != j) ? 1.0 / dij : 0.0;
        ird[k] = (i != j) ? IR / dij : 0.0;
    }
    for (int i = tid; i < S; i += kThreads) {
        se[i] = se_in[i];
        occ[i] = (i < N) ? occ_g[i] : 0;
    }
    __syncthreads();

    const int chunk = (SS + kThreads - 1) / kThreads;
    const int kb = tid * chunk;
    const int ke = min(kb + chunk, SS);
    double time = 0.0;
    int status = KMC_OK;

    for (int64_t hop = 0; hop < hops; ++hop) {
        // site energies
        for (int i = tid; i < N; i += kThreads) {
            double acc = 0.0;
            const double *row = invd + (size_t)i * N;
            for (int j = 0; j < N; ++j)
                if (j != i && !occ[j]) acc += row[j];
            double e = Ec[i];
            e += mIR * acc;
            se[i] = e;
        }
        __syncthreads();
        // rates over this thread's chunk
        double lsum = 0.0;
        for (int k = kb; k < ke; ++k) {
            const int i = k / S, j = k - (k / S) * S;
            double t = 0.0;
            if (possible(i, j, N, occ)) {
                double dE;
                if (i < N && j < N) dE = se[j] - se[i] - ird[(size_t)i * N + j];
                else dE = se[j] - se[i];
                // x / 1.0 == x exactly, so kT = 1 skips the division bit-exactly
                t = (dE > 0) ? nu * exp(kT_is_one ? -dE : -dE / kT) : nu;
            }
            t = tc[k] * t;
            cum[k] = t;
            lsum += t;
        }
        double blocktot;
        const double base = block_exclusive_scan(lsum, red, blocktot);
        if (flux_time) {
            // every rate of this state is in cum (the scan synchronised): the
            // expected net hole flow into each electrode, column N+e minus
            // row N+e, summed in ascending site order
            for (int e = tid; e < P; e += kThreads) {
                double in = 0.0, out = 0.0;
                for (int i = 0; i < N; ++i) in += cum[(size_t)i * S + N + e];
                for (int j = 0; j < N; ++j) out += cum[(size_t)(N + e) * S + j];
                sh_flux[e] = in - out;
            }
            __syncthreads();
        }
        // running sums continued from the chunk's base
        double run = base;
        for (int k = kb; k < ke; ++k) {
            run = (k == 0) ? cum[k] : cum[k] + run;
            cum[k] = run;
        }
        if (ke == SS && kb < ke) sh_total = run;
        if (tid == 0) ev_min = 0x7fffffff;
        __syncthreads();
        const double total = sh_total;
        if (!(total > 0.0) || !(total < 1.0e300)) {
            status = KMC_ERR_NONFINITE;
            break;
        }
        double u1, u2;
        if (uniforms) {
            u1 = uniforms[2 * hop];
            u2 = uniforms[2 * hop + 1];
        } else {
            const u32x4 r = philox4x32_10(u32x4{static_cast<uint32_t>(hop), static_cast<uint32_t>(hop >> 32), 0u, 0u},
                                          static_cast<uint32_t>(seed), static_cast<uint32_t>(seed >> 32));
            u1 = u01_from64(r.x, r.y);
            u2 = u01_from64(r.z, r.w);
        }
        // First k with cum_k/total >= u2 (the reference's test, one FP64
        // division per candidate).  cum is non-decreasing, so only the chunk
        // whose last entry passes can hold it; a chunk whose last entry is
        // below u2*total by far more than the rounding of either side (a
        // relative 1e-12) cannot pass and is skipped without dividing.
        if (kb < ke && !(cum[ke - 1] < u2 * total * (1.0 - 1.0e-12))) {
            for (int k = kb; k < ke; ++k) {
                if (cum[k] / total >= u2) { atomicMin(&ev_min, k); break; }
            }
        }
        __syncthreads();
        if (tid == 0) {
            int ev = ev_min;
            if (ev == 0x7fffffff) ev = 0;   // cannot happen: cum[SS-1]/total == 1 > u2
            const int from = ev / S, to = ev - (ev / S) * S;
            const double scale = 1.0 / total;
            const double hop_time = -log(1.0 - u1) * scale;
            if (from < N) occ[from] = 0; else eo[from - N] -= 1;
            if (to < N) occ[to] = 1; else eo[to - N] += 1;
            if (record) traffic[(size_t)from * S + to] += 1.0;
            if (hop_log) { hop_log[2 * hop] = from; hop_log[2 * hop + 1] = to; }
            if (flux_time)
                for (int e = 0; e < P; ++e) flux_time[e] += sh_flux[e] * hop_time;
            sh_hop_time = hop_time;
        }
        __syncthreads();
        const double hop_time = sh_hop_time;
        if (record)
            for (int i = tid; i < N; i += kThreads)
                if (occ[i]) oit[i] += hop_time;
        time += hop_time;
    }
    for (int i = tid; i < N; i += kThreads) occ_g[i] = occ[i];
    if (tid == 0) {
        *time_out = time;
        *status_out = status;
    }
}

__global__ void __launch_bounds__(kThreads) f64_chain_kernel(
    int N, int P, double nu, double kT, double I0, double R, uint8_t *occ_g, const double *d,
    const double *Ec, const double *se_in, const double *tc, int64_t *eo, int64_t hops,
    int record, double *traffic, double *oit, const double *uniforms, uint64_t seed,
    int32_t *hop_log, double *time_out, int32_t *status_out, double *ws, double *flux_time)
{
    f64_chain(N, P, nu, kT, I0, R, occ_g, d, Ec, se_in, tc, eo, hops, record, traffic, oit, uniforms,
              seed, hop_log, time_out, status_out, ws, flux_time);
}

// Many independent chains in one launch, one block each (Philox streams
// keyed by each chain's own seed).
__global__ void __launch_bounds__(kThreads) f64_batch_kernel(const kmc_f64_batch B, size_t ws_doubles)
{
    const int c = blockIdx.x;
    const int N = B.N[c], P = B.P[c];
    // a chain whose sizes do not fit the launch (shared memory is sized for
    // max_sites, the flux buffer for 64 electrodes) stops before any access
    if (N < 0 || P < 0 || N + P <= 0 || N + P > B.max_sites || (B.flux_time && P > 64) || !(B.kT[c] > 0.0) ||
        B.hops[c] < 0) {
        if (threadIdx.x == 0) {
            B.status_out[c] = KMC_ERR_INVALID;
            B.time_out[c] = 0.0;
        }
        return;
    }
    const int64_t so = B.site_off[c], eo = B.el_off[c], po = B.pair_off[c], vo = B.se_off[c];
    double *fx = B.flux_time ? B.flux_time + eo : nullptr;
    double *tr = B.record ? B.traffic + B.traffic_off[c] : nullptr;
    double *oit = B.record ? B.occupations_in_time + so : nullptr;
    f64_chain(N, P, B.nu[c], B.kT[c], B.I_0[c], B.R[c], B.occupation + so, B.distances + po, B.E_constant + so,
              B.site_energies + vo, B.transitions_constant + po, B.electrode_occupation + eo, B.hops[c],
              B.record, tr, oit, nullptr, B.seeds[c], nullptr, B.time_out + c, B.status_out + c,
              B.workspace + (size_t)c * ws_doubles, fx);
}

}  // namespace

size_t f64_workspace_size(int S)
{
    return sizeof(double) * (2 * (size_t)S * S + (size_t)S * S);
}

int simulate_f64(int N, int P, double nu, double kT, double I0, double R, uint8_t *occ,
                 const double *d, const double *Ec, const double *se, const double *tc,
                 int64_t *eo, int64_t hops, int record, double *traffic, double *oit,
                 const double *uniforms, uint64_t seed, int32_t *hop_log, double *time_out,
                 int32_t *status_out, void *ws, size_t ws_bytes, cudaStream_t st, double *flux_time)
{
    const int S = N + P;
    if (N < 0 || P < 0 || S <= 0 || S > kMaxSitesF64 || hops < 0)
        return fail(KMC_ERR_INVALID, "simulate_f64: bad sizes N=%d P=%d hops=%lld", N, P, (long long)hops);
    if (!occ && N > 0) return fail(KMC_ERR_INVALID, "simulate_f64: occupation is NULL");
    if (!d || !Ec || !se || !tc || (!eo && P > 0) || !time_out || !status_out || !ws)
        return fail(KMC_ERR_INVALID, "simulate_f64: a required pointer is NULL");
    if (record && (!traffic || (!oit && N > 0)))
        return fail(KMC_ERR_INVALID, "simulate_f64: record needs traffic and occupations_in_time");
    if (ws_bytes < f64_workspace_size(S))
        return fail(KMC_ERR_INVALID, "simulate_f64: workspace %zu bytes < %zu", ws_bytes, f64_workspace_size(S));
    if (!(kT > 0)) return fail(KMC_ERR_INVALID, "simulate_f64: kT must be positive");
    if (flux_time && P > 64) return fail(KMC_ERR_INVALID, "simulate_f64: flux_time supports at most 64 electrodes");
    const size_t smem = sizeof(double) * (S + 32) + S + 16;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(f64_chain_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(smem));
        if (e != cudaSuccess) return fail_cuda(e, "cudaFuncSetAttribute(f64)");
    }
    f64_chain_kernel<<<1, kThreads, smem, st>>>(N, P, nu, kT, I0, R, occ, d, Ec, se, tc, eo, hops,
                                                record, traffic, oit, uniforms, seed, hop_log,
                                                time_out, status_out, static_cast<double *>(ws), flux_time);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail_cuda(e, "f64 launch");
    return KMC_OK;
}


size_t f64_batch_workspace_size(int n_chains, int max_sites)
{
    return (size_t)n_chains * f64_workspace_size(max_sites);
}

int simulate_f64_batch(const kmc_f64_batch &B, cudaStream_t st)
{
    if (B.n_chains < 0 || B.max_sites <= 0 || B.max_sites > kMaxSitesF64)
        return fail(KMC_ERR_INVALID, "simulate_f64_batch: bad sizes (n_chains %d, max_sites %d)", B.n_chains,
                    B.max_sites);
    if (B.n_chains == 0) return KMC_OK;
    if (!B.N || !B.P || !B.nu || !B.kT || !B.I_0 || !B.R || !B.pair_off || !B.distances ||
        !B.transitions_constant || !B.site_off || !B.E_constant || !B.se_off || !B.site_energies ||
        !B.occupation || !B.el_off || !B.electrode_occupation || !B.hops || !B.seeds || !B.time_out ||
        !B.status_out || !B.workspace)
        return fail(KMC_ERR_INVALID, "simulate_f64_batch: a required pointer is NULL");
    if (B.record && (!B.traffic || !B.traffic_off || !B.occupations_in_time))
        return fail(KMC_ERR_INVALID, "simulate_f64_batch: record needs traffic, traffic_off, occupations_in_time");
    if (B.workspace_bytes < f64_batch_workspace_size(B.n_chains, B.max_sites))
        return fail(KMC_ERR_INVALID, "simulate_f64_batch: workspace %zu bytes < %zu", B.workspace_bytes,
                    f64_batch_workspace_size(B.n_chains, B.max_sites));
    // per-chain sizes are checked by each block (KMC_ERR_INVALID in status_out)
    const int S = B.max_sites;
    const size_t smem = sizeof(double) * (S + 32) + S + 16;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(f64_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(smem));
        if (e != cudaSuccess) return fail_cuda(e, "cudaFuncSetAttribute(f64 batch)");
    }
    f64_batch_kernel<<<B.n_chains, kThreads, smem, st>>>(B, f64_workspace_size(S) / sizeof(double));
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? KMC_OK : fail_cuda(e, "f64 batch launch");
}

// ---------------------------------------------------------------------------
// Allocation-free variant
//
// Some callers of this kernel cannot allocate device memory when they call
// it: a host that owns every byte of the device through its own memory pool
// and hands plugins only the buffers it placed, or a latency-bound loop in
// which a cudaMalloc / cudaFree (which may synchronise the whole device)
// would stall other work.  For them the workspace is a fixed array in this
// library's device memory instead of a caller-provided buffer.
// ---------------------------------------------------------------------------

// Largest network the static workspace holds: S = N + P <= 128 sites, i.e.
// 3 * 128^2 doubles = 384 KiB, resident on every device that loads the
// library until the process exits.
constexpr int kStaticWorkspaceSites = 128;
static __device__ __align__(256) double g_f64_static_workspace[3 * kStaticWorkspaceSites * kStaticWorkspaceSites];

// Device address of the static workspace in the current context.  The
// array's name is only a host-side stand-in in host code, so its address is
// looked up on every call (cheap once the module is loaded).  It is not
// cached: after a cudaDeviceReset, or in another context on the same device,
// the module is loaded again at a different address.
static int static_workspace(double **out)
{
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_f64_static_workspace);
    if (e != cudaSuccess) return fail_cuda(e, "simulate_f64_static: cudaGetSymbolAddress");
    *out = static_cast<double *>(p);
    return KMC_OK;
}

}  // namespace kmc

extern "C" int kmc_simulate_f64_static(int32_t n_acceptors, int32_t n_electrodes, double nu,
                                       double kT, double I_0, double R, uint8_t *occupation,
                                       const double *distances, const double *E_constant,
                                       const double *site_energies,
                                       const double *transitions_constant,
                                       int64_t *electrode_occupation, int64_t hops, int32_t record,
                                       double *traffic, double *occupations_in_time,
                                       const double *uniforms, uint64_t seed, int32_t *hop_log,
                                       double *time_out, int32_t *status_out, void *stream)
{
    using namespace kmc;
    const int S = n_acceptors + n_electrodes;
    if (n_acceptors < 0 || n_electrodes < 0 || S <= 0 || S > kStaticWorkspaceSites)
        return fail(KMC_ERR_INVALID,
                    "kmc_simulate_f64_static: %d sites (N=%d, P=%d); the fixed workspace holds at most %d "
                    "(use kmc_simulate_f64 with a caller workspace for larger networks)",
                    S, n_acceptors, n_electrodes, kStaticWorkspaceSites);
    double *ws = nullptr;
    const int rc = static_workspace(&ws);
    if (rc != KMC_OK) return rc;
    // The kernel writes every workspace entry it reads within the call
    // (1/d, I_0 R/d and the running sums), so the contents a previous call
    // left behind need no clearing.
    return simulate_f64(n_acceptors, n_electrodes, nu, kT, I_0, R, occupation, distances, E_constant,
                        site_energies, transitions_constant, electrode_occupation, hops, record,
                        traffic, occupations_in_time, uniforms, seed, hop_log, time_out, status_out,
                        ws, sizeof(double) * 3 * (size_t)kStaticWorkspaceSites * kStaticWorkspaceSites,
                        static_cast<cudaStream_t>(stream), nullptr);
}

namespace kmc {

int preload_f64()
{
    int rc;
    if ((rc = touch_kernel(f64_chain_kernel)) != KMC_OK) return rc;
    return touch_kernel(f64_batch_kernel);
}

}  // namespace kmc
