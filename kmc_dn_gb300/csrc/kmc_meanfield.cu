// kmc_meanfield.cu -- mean-field relaxation of a batch of networks (the Go
// library's probSimulate, goSimulation/probabilitySimulation.go:53-157).
//
// State per network: the occupation probability of every acceptor.  One
// iteration (the Go loop's "hop"):
//   energies  e_i = Ec_i - I_0 R sum_{j != i} (1 - o_j) / d_ij        (:85-94)
//   rates     t_ij = w_ij nu tc_ij exp(-max(dE_ij, 0) / kT), the weight
//             w_ij the probability that the transition is possible:
//             (1 - o_j) o_i between acceptors, o_i into an electrode,
//             1 - o_j out of one, 0 between electrodes             (:7-49)
//   step      the largest fraction m <= 1 of the expected flow that keeps
//             every o_i in [0, 1]; time += 0.98 m / sum t           (:95-110)
//   apply     o_i += m (in_i - out_i) / sum t, the electrodes' counters
//             likewise; clamp to [0, 1]                            (:118-152)
//
// One block of 128 threads per network; the pair tables (K = nu tc,
// B = I_0 R / d) and the iteration's S x S rates live in shared memory, so
// an iteration touches no global memory outside record mode.  A thread per
// acceptor sums its energy, a thread per pair evaluates a rate, a thread per
// site sums its row (outflow) or its column (inflow) in a fixed order, so a
// run is deterministic and a network's result does not depend on the batch.
// Two rate precisions:
//   KMC_MF_RATES_F64  everything in FP64, exp() per pair (the reference's
//                     arithmetic up to rounding order),
//   KMC_MF_RATES_F32  FP32 energies and rates (one ex2.approx per pair),
//                     compensated FP32 row/column sums, FP64 state, step
//                     and clock: GB300 runs FP64 at 1/64 of FP32, so only
//                     O(S) FP64 work per iteration remains.
// No spin-waits; every loop is bounded by the iteration count or S.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>

#include "kmc_internal.h"

namespace kmc {
namespace {

constexpr int kMfThreads = 128;
constexpr int kMfSmemLimit = 226 * 1024;   // dynamic; leaves room for the static words

__device__ __forceinline__ double warp_sum(double x)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
}

__device__ __forceinline__ double warp_min(double x)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x = fmin(x, __shfl_xor_sync(0xffffffffu, x, o));
    return x;
}

__device__ __forceinline__ float ex2_approx(float x)
{
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

template <bool F64> struct MfTypes;
template <> struct MfTypes<true> { using Real = double; using Pair = double2; };
template <> struct MfTypes<false> { using Real = float; using Pair = float2; };

// Running sum of one thread: plain FP64, or in FP32 as an unevaluated pair
// (hi, lo) updated by TwoSum (Knuth), six FP32 operations per term, which
// keeps the sum of FP32 terms to about 2^-44 relative without the FP64
// pipe.
// Two-float arithmetic for the FP32-rate mode's flows: TwoSum, and a sum
// normalised so that |lo| <= ulp(hi) / 2.
struct F2 {
    float hi, lo;
};
__device__ __forceinline__ F2 df_add(F2 x, F2 y)
{
    const float s = __fadd_rn(x.hi, y.hi);
    const float bp = __fsub_rn(s, x.hi);
    const float e = __fadd_rn(__fsub_rn(x.hi, __fsub_rn(s, bp)), __fsub_rn(y.hi, bp));
    const float lo = __fadd_rn(e, __fadd_rn(x.lo, y.lo));
    const float hi = __fadd_rn(s, lo);
    return F2{hi, __fsub_rn(lo, __fsub_rn(hi, s))};
}
__device__ __forceinline__ F2 warp_sum_df(F2 x)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        x = df_add(x, F2{__shfl_xor_sync(0xffffffffu, x.hi, o), __shfl_xor_sync(0xffffffffu, x.lo, o)});
    return x;
}
__device__ __forceinline__ float warp_min_f(float x)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x = fminf(x, __shfl_xor_sync(0xffffffffu, x, o));
    return x;
}

template <bool F64> struct Acc;
template <> struct Acc<true> {
    double s = 0.0;
    __device__ __forceinline__ void add(double x) { s += x; }
    __device__ __forceinline__ double value() const { return s; }
};
template <> struct Acc<false> {
    float hi = 0.0f, lo = 0.0f;
    __device__ __forceinline__ void add(float x)
    {
        const float t = __fadd_rn(hi, x);
        const float bp = __fsub_rn(t, hi);
        const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(t, bp)), __fsub_rn(x, bp));
        hi = t;
        lo = __fadd_rn(lo, err);
    }
    __device__ __forceinline__ double value() const { return static_cast<double>(hi) + static_cast<double>(lo); }
    __device__ __forceinline__ F2 pair() const { return F2{hi, lo}; }
};

// Row stride of the shared S x S arrays: odd, so that a thread per row
// reading along its row and a thread per column reading down it both hit
// distinct banks.
__device__ __host__ __forceinline__ int row_stride(int S) { return S | 1; }

}  // namespace

size_t mf_smem_bytes(int S, int rates)
{
    const size_t pairs = static_cast<size_t>(S) * row_stride(S);
    const size_t per_pair = rates == KMC_MF_RATES_F64 ? 16 + 8 : 8 + 4;
    // occ, out, in, avg, eo (double) + e (Real) + occ, e (float) per site, + scalars
    return pairs * per_pair + static_cast<size_t>(S) * (6 * 8 + 2 * 4) + 64;
}

namespace {

template <bool F64>
__global__ void __launch_bounds__(kMfThreads, F64 ? 4 : 8) mf_kernel(kmc_mf_batch b)
{
    using Real = typename MfTypes<F64>::Real;
    using Pair = typename MfTypes<F64>::Pair;
    extern __shared__ __align__(16) unsigned char smem[];
    const int c = blockIdx.x;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int N = b.N[c], P = b.P[c], S = N + P;
    const int SS = S * S;
    const int SP = row_stride(S);
    if (S < 1 || S > b.max_sites) {
        if (tid == 0 && b.status) b.status[c] = KMC_ERR_INVALID;
        return;
    }
    const double nu = b.nu[c], kT = b.kT[c], I0R = b.I_0[c] * b.R[c];
    const double *dist = b.distances + b.pair_off[c];
    const double *tcon = b.transitions_constant + b.pair_off[c];
    const double *Ec = b.E_constant + b.site_off[c];
    double *se_out = b.site_energies + b.site_off[c];
    double *occ_io = b.occupation + b.site_off[c];

    // shared-memory carve (8-byte items first); S x S arrays use row stride SP
    Pair *KB = reinterpret_cast<Pair *>(smem);
    Real *rt = reinterpret_cast<Real *>(KB + S * SP);
    double *occ = reinterpret_cast<double *>(
        (reinterpret_cast<uintptr_t>(rt + S * SP) + 15) & ~static_cast<uintptr_t>(15));
    double *outs = occ + S;
    double *ins = outs + S;
    double *avg = ins + S;
    double *eo = avg + S;
    Real *e = reinterpret_cast<Real *>(eo + S);   // site energies (electrodes: voltages)
    float *of = reinterpret_cast<float *>(e + S);  // FP32 copy of the probabilities
    __shared__ double sh_f, sh_ts, sh_time;
    __shared__ int sh_stop;

    // pair tables: K = nu*tc, B = I_0 R / d between acceptors (0 otherwise)
    for (int p = tid; p < SS; p += kMfThreads) {
        const int i = p / S, j = p - (p / S) * S;
        const double K = nu * tcon[p];
        const double B = (i < N && j < N) ? I0R / dist[p] : 0.0;
        KB[i * SP + j] = Pair{static_cast<Real>(K), static_cast<Real>(B)};
    }
    for (int k = tid; k < S; k += kMfThreads) {
        occ[k] = k < N ? occ_io[k] : 0.0;
        of[k] = static_cast<float>(occ[k]);
        e[k] = k < N ? Real(0) : static_cast<Real>(se_out[k]);
        avg[k] = (b.record && k < N) ? b.average_occupation[b.site_off[c] + k] : 0.0;
        eo[k] = 0.0;
    }
    if (tid == 0) { sh_time = 0.0; sh_stop = 0; }
    __syncthreads();

    const Real ec_i = tid < N ? static_cast<Real>(Ec[tid]) : Real(0);
    const double inv_kT = 1.0 / kT;
    const float c2 = static_cast<float>(1.4426950408889634 / kT);
    const int64_t hops = b.hops[c];
    double *traffic = b.record ? b.traffic + b.traffic_off[c] : nullptr;
    int64_t it = 0;
    for (; it < hops; ++it) {
        // (1) energies from the probabilities, a thread per acceptor
        for (int i = tid; i < N; i += kMfThreads) {
            Real acc = 0;
            for (int j = 0; j < N; ++j) {
                const Real w = F64 ? static_cast<Real>(1.0 - occ[j]) : static_cast<Real>(1.0f - of[j]);
                if (j != i) acc += w * KB[i * SP + j].y;
            }
            e[i] = (i == tid ? ec_i : static_cast<Real>(Ec[i])) - acc;
        }
        __syncthreads();

        // (2) the S x S expected rates, a thread per pair
        for (int p = tid; p < SS; p += kMfThreads) {
            const int i = p / S, j = p - (p / S) * S;
            const Pair kb = KB[i * SP + j];
            Real r;
            if (F64) {
                double w;
                if (i >= N && j >= N) w = 0.0;
                else if (i >= N) w = 1.0 - occ[j];
                else if (j >= N) w = occ[i];
                else w = (1.0 - occ[j]) * occ[i];
                const double dE = static_cast<double>(e[j]) - static_cast<double>(e[i]) - static_cast<double>(kb.y);
                r = static_cast<Real>(w * static_cast<double>(kb.x) * exp(-fmax(dE, 0.0) * inv_kT));
            } else {
                float w;
                if (i >= N && j >= N) w = 0.0f;
                else if (i >= N) w = 1.0f - of[j];
                else if (j >= N) w = of[i];
                else w = (1.0f - of[j]) * of[i];
                const float dE = static_cast<float>(e[j]) - static_cast<float>(e[i]) - static_cast<float>(kb.y);
                r = static_cast<Real>(w * static_cast<float>(kb.x) * ex2_approx(-c2 * fmaxf(dE, 0.0f)));
            }
            rt[i * SP + j] = r;
        }
        __syncthreads();

        // (3) outflows (threads 0..S-1, along rows) and inflows (threads
        // S..2S-1, down columns), each a sequential sum in a fixed order
        // (FP32-rate mode: kept as two-float pairs in the same slots)
        for (int q = tid; q < 2 * S; q += kMfThreads) {
            Acc<F64> a;
            const int k = q < S ? q : q - S;
            if (q < S) {
                for (int j = 0; j < S; ++j) a.add(rt[q * SP + j]);
            } else {
                for (int i = 0; i < S; ++i) a.add(rt[i * SP + k]);
            }
            double *dst = q < S ? outs : ins;
            if constexpr (F64) dst[k] = a.value();
            else reinterpret_cast<F2 *>(dst)[k] = a.pair();
        }
        __syncthreads();

        if constexpr (!F64) {
            // (4') total and step size in FP32 / two-float (one warp)
            const F2 *outs2 = reinterpret_cast<const F2 *>(outs);
            const F2 *ins2 = reinterpret_cast<const F2 *>(ins);
            if (warp == 0) {
                F2 tot{0.0f, 0.0f};
                for (int k = lane; k < S; k += 32) tot = df_add(tot, outs2[k]);
                tot = warp_sum_df(tot);
                const float inv = 1.0f / tot.hi;
                float mc = 1.0f;
                for (int k = lane; k < N; k += 32) {
                    const float q = df_add(ins2[k], F2{-outs2[k].hi, -outs2[k].lo}).hi * inv;
                    const float o = of[k];
                    const float nv = o + q;
                    if (nv < 0.0f) mc = fminf(mc, o / -q);
                    if (nv > 1.0f) mc = fminf(mc, (1.0f - o) / q);
                }
                mc = warp_min_f(mc);
                if (lane == 0) {
                    if (!(tot.hi > 0.0f) || !(tot.hi <= 3.0e38f)) {
                        sh_stop = 1;
                    } else {
                        const float ff = mc * inv, tsf = 0.98f * mc * inv;
                        sh_f = ff;
                        sh_ts = tsf;
                        sh_time += static_cast<double>(tsf);
                    }
                }
            }
            __syncthreads();
            if (sh_stop) break;
            // (5') move the expected charge (the state stays FP64), record, clamp
            const float f = static_cast<float>(sh_f);
            for (int k = tid; k < S; k += kMfThreads) {
                const double d = static_cast<double>(df_add(ins2[k], F2{-outs2[k].hi, -outs2[k].lo}).hi * f);
                if (k < N) {
                    if (b.record) avg[k] += occ[k] * sh_ts;
                    const double o = fmin(fmax(occ[k] + d, 0.0), 1.0);
                    occ[k] = o;
                    of[k] = static_cast<float>(o);
                } else {
                    eo[k] += d;
                }
            }
            if (traffic)
                for (int p = tid; p < SS; p += kMfThreads) {
                    const int i = p / S, j = p - (p / S) * S;
                    if (i >= N && j >= N) continue;
                    traffic[p] += static_cast<double>((rt[i * SP + j] - rt[j * SP + i]) * f);
                }
            __syncthreads();
            continue;
        }

        // (4) total and step size (one warp; one FP64 division per iteration)
        if (warp == 0) {
            double tot = 0.0;
            for (int k = lane; k < S; k += 32) tot += outs[k];
            tot = warp_sum(tot);
            const double inv = 1.0 / tot;
            double mc = 1.0;
            for (int k = lane; k < N; k += 32) {
                const double q = (ins[k] - outs[k]) * inv;
                const double nv = occ[k] + q;
                if (nv < 0) mc = fmin(mc, occ[k] / -q);
                if (nv > 1) mc = fmin(mc, (1.0 - occ[k]) / q);
            }
            mc = warp_min(mc);
            if (lane == 0) {
                if (!(tot > 0.0) || !(tot < 1.0e300)) {
                    sh_stop = 1;
                } else {
                    sh_f = mc * inv;              // fraction of each expected flow moved
                    sh_ts = 0.98 * mc * inv;      // time step
                    sh_time += sh_ts;
                }
            }
        }
        __syncthreads();
        if (sh_stop) break;

        // (5) move the expected charge, record, clamp
        const double f = sh_f;
        const double ts = sh_ts;
        for (int k = tid; k < S; k += kMfThreads) {
            const double net = ins[k] - outs[k];
            if (k < N) {
                if (b.record) avg[k] += occ[k] * ts;
                double o = occ[k] + net * f;
                o = o < 0.0 ? 0.0 : (o > 1.0 ? 1.0 : o);
                occ[k] = o;
                of[k] = static_cast<float>(o);
            } else {
                eo[k] += net * f;
            }
        }
        if (traffic)
            for (int p = tid; p < SS; p += kMfThreads) {
                const int i = p / S, j = p - (p / S) * S;
                if (i >= N && j >= N) continue;
                traffic[p] += (static_cast<double>(rt[i * SP + j]) - static_cast<double>(rt[j * SP + i])) * f;
            }
        __syncthreads();
    }

    // outputs
    for (int k = tid; k < S; k += kMfThreads) {
        if (k < N) {
            occ_io[k] = occ[k];
            se_out[k] = static_cast<double>(e[k]);
            if (b.record) b.average_occupation[b.site_off[c] + k] = avg[k];
        } else {
            b.electrode_occupation[b.el_off[c] + (k - N)] = eo[k];
        }
    }
    if (tid == 0) {
        b.time[c] = sh_time;
        if (b.status) b.status[c] = sh_stop ? KMC_ERR_NONFINITE : KMC_OK;
        if (b.iterations_done) b.iterations_done[c] = it;
    }
}

}  // namespace
}  // namespace kmc

using namespace kmc;

extern "C" size_t kmc_mf_smem_bytes(int32_t max_sites, int32_t rates)
{
    if (max_sites < 1) return 0;
    return mf_smem_bytes(max_sites, rates);
}

extern "C" int32_t kmc_mf_max_sites(int32_t rates)
{
    int S = 1;
    while (mf_smem_bytes(S + 1, rates) <= static_cast<size_t>(kMfSmemLimit)) ++S;
    return S;
}

extern "C" int kmc_mf_run(const kmc_mf_batch *b, void *stream)
{
    if (!b) return fail(KMC_ERR_INVALID, "mf_run: NULL batch");
    if (b->n_chains == 0) return KMC_OK;
    if (b->n_chains < 0) return fail(KMC_ERR_INVALID, "mf_run: n_chains < 0");
    if (b->rates != KMC_MF_RATES_F64 && b->rates != KMC_MF_RATES_F32)
        return fail(KMC_ERR_INVALID, "mf_run: rates must be KMC_MF_RATES_F64 or KMC_MF_RATES_F32");
    const int lim = kmc_mf_max_sites(b->rates);
    if (b->max_sites < 1 || b->max_sites > lim)
        return fail(KMC_ERR_INVALID, "mf_run: max_sites %d outside [1, %d] for this rate precision",
                    b->max_sites, lim);
    if (!b->N || !b->P || !b->nu || !b->kT || !b->I_0 || !b->R || !b->pair_off || !b->distances ||
        !b->transitions_constant || !b->site_off || !b->E_constant || !b->site_energies ||
        !b->occupation || !b->el_off || !b->electrode_occupation || !b->hops || !b->time)
        return fail(KMC_ERR_INVALID, "mf_run: NULL array");
    if (b->record && (!b->traffic || !b->traffic_off || !b->average_occupation))
        return fail(KMC_ERR_INVALID, "mf_run: record needs traffic, traffic_off and average_occupation");
    const size_t smem = mf_smem_bytes(b->max_sites, b->rates);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e;
    if (b->rates == KMC_MF_RATES_F64) {
        e = cudaFuncSetAttribute(mf_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        if (e != cudaSuccess) return fail_cuda(e, "mf_run smem attribute");
        mf_kernel<true><<<b->n_chains, kMfThreads, smem, st>>>(*b);
    } else {
        e = cudaFuncSetAttribute(mf_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        if (e != cudaSuccess) return fail_cuda(e, "mf_run smem attribute");
        mf_kernel<false><<<b->n_chains, kMfThreads, smem, st>>>(*b);
    }
    e = cudaGetLastError();
    return e == cudaSuccess ? KMC_OK : fail_cuda(e, "mf_run launch");
}

namespace {

// Device copy of a host array, freed on scope exit.
struct DevBuf {
    void *p = nullptr;
    ~DevBuf() { if (p) cudaFree(p); }
};

template <typename T>
int upload(DevBuf &d, const T *h, int64_t n, cudaStream_t st, bool copy = true)
{
    if (!h || n <= 0) return KMC_OK;
    cudaError_t e = cudaMalloc(&d.p, sizeof(T) * static_cast<size_t>(n));
    if (e != cudaSuccess) return fail(KMC_ERR_OOM, "mf_run_host: device allocation of %lld bytes failed",
                                      (long long)(sizeof(T) * n));
    if (copy) {
        e = cudaMemcpyAsync(d.p, h, sizeof(T) * static_cast<size_t>(n), cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) return fail_cuda(e, "mf_run_host upload");
    }
    return KMC_OK;
}

template <typename T>
int download(T *h, const DevBuf &d, int64_t n, cudaStream_t st)
{
    if (!h || !d.p || n <= 0) return KMC_OK;
    cudaError_t e = cudaMemcpyAsync(h, d.p, sizeof(T) * static_cast<size_t>(n), cudaMemcpyDeviceToHost, st);
    return e == cudaSuccess ? KMC_OK : fail_cuda(e, "mf_run_host download");
}

}  // namespace

// Same batch with HOST pointers: sizes follow from the offsets, device
// copies live for the call, results are copied back before it returns.
extern "C" int kmc_mf_run_host(const kmc_mf_batch *h, void *stream)
{
    if (!h) return fail(KMC_ERR_INVALID, "mf_run_host: NULL batch");
    const int n = h->n_chains;
    if (n == 0) return KMC_OK;
    if (n < 0 || !h->N || !h->P || !h->pair_off || !h->site_off || !h->el_off || !h->hops)
        return fail(KMC_ERR_INVALID, "mf_run_host: bad chain arrays");
    if (h->record && !h->traffic_off) return fail(KMC_ERR_INVALID, "mf_run_host: record needs traffic_off");
    int64_t n_pairs = 0, n_sites = 0, n_el = 0, n_tr = 0;
    for (int c = 0; c < n; ++c) {
        const int64_t S = static_cast<int64_t>(h->N[c]) + h->P[c];
        if (h->N[c] < 0 || h->P[c] < 0 || S < 1 || h->pair_off[c] < 0 || h->site_off[c] < 0 ||
            h->el_off[c] < 0 || (h->record && h->traffic_off[c] < 0))
            return fail(KMC_ERR_INVALID, "mf_run_host: chain %d has bad sizes or offsets", c);
        n_pairs = std::max(n_pairs, h->pair_off[c] + S * S);
        n_sites = std::max(n_sites, h->site_off[c] + S);
        n_el = std::max(n_el, h->el_off[c] + h->P[c]);
        if (h->record) n_tr = std::max(n_tr, h->traffic_off[c] + S * S);
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    DevBuf dN, dP, dnu, dkT, dI0, dR, dpo, dd, dtc, dso, dEc, dse, docc, deo_off, deo, dh, dto, dtr, davg,
        dtime, dst, dit;
    int rc;
#define KMC_UP(buf, ptr, cnt) if ((rc = upload(buf, ptr, cnt, st)) != KMC_OK) return rc
    KMC_UP(dN, h->N, n); KMC_UP(dP, h->P, n); KMC_UP(dnu, h->nu, n); KMC_UP(dkT, h->kT, n);
    KMC_UP(dI0, h->I_0, n); KMC_UP(dR, h->R, n); KMC_UP(dpo, h->pair_off, n);
    KMC_UP(dd, h->distances, n_pairs); KMC_UP(dtc, h->transitions_constant, n_pairs);
    KMC_UP(dso, h->site_off, n); KMC_UP(dEc, h->E_constant, n_sites); KMC_UP(dse, h->site_energies, n_sites);
    KMC_UP(docc, h->occupation, n_sites); KMC_UP(deo_off, h->el_off, n); KMC_UP(dh, h->hops, n);
    if (h->record) {
        KMC_UP(dto, h->traffic_off, n); KMC_UP(dtr, h->traffic, n_tr);
        KMC_UP(davg, h->average_occupation, n_sites);
    }
#undef KMC_UP
    if ((rc = upload(deo, h->electrode_occupation, std::max<int64_t>(n_el, 1), st, false)) != KMC_OK) return rc;
    if ((rc = upload(dtime, h->time, n, st, false)) != KMC_OK) return rc;
    if ((rc = upload(dst, h->status, n, st, false)) != KMC_OK) return rc;
    if ((rc = upload(dit, h->iterations_done, n, st, false)) != KMC_OK) return rc;
    kmc_mf_batch d = *h;
    d.N = static_cast<const int32_t *>(dN.p); d.P = static_cast<const int32_t *>(dP.p);
    d.nu = static_cast<const double *>(dnu.p); d.kT = static_cast<const double *>(dkT.p);
    d.I_0 = static_cast<const double *>(dI0.p); d.R = static_cast<const double *>(dR.p);
    d.pair_off = static_cast<const int64_t *>(dpo.p);
    d.distances = static_cast<const double *>(dd.p);
    d.transitions_constant = static_cast<const double *>(dtc.p);
    d.site_off = static_cast<const int64_t *>(dso.p);
    d.E_constant = static_cast<const double *>(dEc.p);
    d.site_energies = static_cast<double *>(dse.p);
    d.occupation = static_cast<double *>(docc.p);
    d.el_off = static_cast<const int64_t *>(deo_off.p);
    d.electrode_occupation = static_cast<double *>(deo.p);
    d.hops = static_cast<const int64_t *>(dh.p);
    d.traffic_off = static_cast<const int64_t *>(dto.p);
    d.traffic = static_cast<double *>(dtr.p);
    d.average_occupation = static_cast<double *>(davg.p);
    d.time = static_cast<double *>(dtime.p);
    d.status = static_cast<int32_t *>(dst.p);
    d.iterations_done = static_cast<int64_t *>(dit.p);
    if ((rc = kmc_mf_run(&d, stream)) != KMC_OK) return rc;
    if ((rc = download(h->occupation, docc, n_sites, st)) != KMC_OK) return rc;
    if ((rc = download(h->site_energies, dse, n_sites, st)) != KMC_OK) return rc;
    if ((rc = download(h->electrode_occupation, deo, n_el, st)) != KMC_OK) return rc;
    if ((rc = download(h->time, dtime, n, st)) != KMC_OK) return rc;
    if ((rc = download(h->status, dst, n, st)) != KMC_OK) return rc;
    if ((rc = download(h->iterations_done, dit, n, st)) != KMC_OK) return rc;
    if (h->record) {
        if ((rc = download(h->traffic, dtr, n_tr, st)) != KMC_OK) return rc;
        if ((rc = download(h->average_occupation, davg, n_sites, st)) != KMC_OK) return rc;
    }
    cudaError_t e = cudaStreamSynchronize(st);
    return e == cudaSuccess ? KMC_OK : fail_cuda(e, "mf_run_host");
}

namespace kmc {

int preload_meanfield()
{
    int rc;
    if ((rc = touch_kernel(mf_kernel<true>)) != KMC_OK) return rc;
    return touch_kernel(mf_kernel<false>);
}

}  // namespace kmc
