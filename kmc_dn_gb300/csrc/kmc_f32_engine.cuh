// kmc_f32_engine.cuh -- batched FP32 hop-loop engine for sm_103a (the
// kernels; kmc_f32_*.cu instantiate them, kmc_f32.cu validates and
// dispatches a launch).
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
//               lists (d from one rsqrt; no table traffic; block groups
//               keep the target list in component-wise pairs and evaluate
//               two targets of a row with packed FP32x2 arithmetic).
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
#pragma once
#include <cstdint>
#include <cstdio>
#include <cuda_runtime.h>

#include "kmc_common.cuh"
#include "kmc_internal.h"

namespace kmc {
namespace {


constexpr float kLog2e = 1.4426950408889634f;
constexpr int kMaxElectrodes = 64;
// Debug builds (-DKMC_DEBUG_CHECKS) check the hop loop's decoded pair and
// list indices once per hop outside the pair walk; a violation stops the
// chain with KMC_ERR_INVALID before the index is used.  Release builds
// compile the checks away.
#ifdef KMC_DEBUG_CHECKS
#define KMC_DCHECK(cond) do { if (!(cond)) dbg_bad = 1; } while (0)
#else
#define KMC_DCHECK(cond) do { } while (0)
#endif

// Section-clock builds (-DKMC_SECTION_CLOCKS) time the phases of every hop
// with the SM clock; the group's thread 0 adds its per-phase cycle counts and
// hop count to kSectionSlots device counters at the end of each launch
// (kmc_section_clocks reads them).  Release builds compile them away.
#ifdef KMC_SECTION_CLOCKS
constexpr int kSections = 8;   // top, pairs, uniforms, scan, search, clock, rebuild, update
// one set per translation unit that instantiates kernels; kmc_section_clocks
// sums them
__device__ unsigned long long g_section_clocks[kSections + 1];

// Add this translation unit's counters to out (and zero them with reset).
inline int section_clocks_read(uint64_t *out, int reset)
{
    unsigned long long v[kSections + 1];
    cudaError_t e = cudaMemcpyFromSymbol(v, g_section_clocks, sizeof(v));
    if (e != cudaSuccess) return fail_cuda(e, "section_clocks read");
    for (int k = 0; k <= kSections; ++k) out[k] += v[k];
    if (reset) {
        const unsigned long long z[kSections + 1] = {};
        e = cudaMemcpyToSymbol(g_section_clocks, z, sizeof(z));
        if (e != cudaSuccess) return fail_cuda(e, "section_clocks reset");
    }
    return KMC_OK;
}
#define KMC_SECTION(k)                                                   \
    do {                                                                 \
        const uint32_t t_ = static_cast<uint32_t>(clock());              \
        sec_cycles[k] += t_ - sec_last;                                  \
        sec_last = t_;                                                   \
    } while (0)
#else
#define KMC_SECTION(k) do { } while (0)
#endif

#ifndef KMC_PAIR_UNROLL
#define KMC_PAIR_UNROLL 4
#endif
// Unroll of the pair walk (four steps = eight pairs in flight per thread):
// on the N=30 ensemble 10 % faster than no unrolling and 5 % faster than two
// steps; the large networks are insensitive to it.  Steps of four or eight
// pairs with all their loads issued before the running-sum stores measured
// 1-2.5 % slower than two-pair steps.
constexpr int kPairUnroll = KMC_PAIR_UNROLL;

// a compile-time bool as a type (selects a lambda's instantiation)
template <bool V>
struct BoolC {
    static constexpr bool value = V;
};

__device__ __forceinline__ float ex2_approx(float x)
{
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ float rcp_approx(float x)
{
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Nanosecond wall clock of the GPU (PTX %globaltimer).
__device__ __forceinline__ uint64_t globaltimer_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ float rsqrt_approx(float x)
{
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// ---------------------------------------------------------------------------
// Two-float values hi + lo and TwoSum (Knuth): the exact rounding error of a
// float add, used to carry the site energies compensated.
// ---------------------------------------------------------------------------
struct F2 {
    float hi, lo;
};

__device__ __forceinline__ F2 two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bp = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp));
    return F2{s, e};
}

// hi + lo += c: the rounding error of the high-part add (TwoSum) goes to the
// low part, so a long series of increments keeps its exact sum to ~2^-47
// instead of accumulating one rounding per increment.
__device__ __forceinline__ void comp_add(float &hi, float &lo, float c)
{
    const F2 s = two_sum(hi, c);
    hi = s.hi;
    lo = __fadd_rn(lo, s.lo);
}





// ---------------------------------------------------------------------------
// Exact fixed-point selection.  The per-thread FP32 sums of a group are
// converted to 64-bit integers on a common power-of-two scale set by the
// largest of them (24 mantissa bits shifted left by kShift, so the group's
// total stays below 2^62), scanned with integer adds, which are exact, and
// compared with u * total computed exactly from a 64-bit fixed-point u.  The
// comparison is therefore exact for the FP32 per-thread sums it is given:
// finer than an FP64 compare, on the integer pipe.  Only a thread's own sum
// below 2^-(23 + kShift) of the largest one is truncated (at most 2^-52 of
// the total).
// ---------------------------------------------------------------------------
template <int G>
struct FixShift {
    static constexpr int kLog = G <= 4 ? 2 : G <= 8 ? 3 : G <= 16 ? 4 : G <= 32 ? 5 : G <= 64 ? 6 :
                                G <= 128 ? 7 : G <= 256 ? 8 : 9;
    static constexpr int kShift = 38 - kLog;   // 24 + kShift + log2(G) = 62
};

// v >= 0 (a sum of ex2 results) on the scale whose unit is
// 2^(emax - 150 - shift), emax the biased exponent of the group's largest sum.
__device__ __forceinline__ uint64_t to_fixed(float v, int emax, int shift)
{
    const uint32_t bits = __float_as_uint(v);
    const int e = static_cast<int>(bits >> 23);
    const uint64_t m = e ? static_cast<uint64_t>((bits & 0x7fffffu) | 0x800000u) : 0ull;
    const int sh = e - emax + shift;
    return sh >= 0 ? (m << sh) : (sh > -24 ? (m >> -sh) : 0ull);
}

// An integer on that scale back to FP32: x * 2^(emax - 150 - shift), as
// (x * 2^-64) * 2^(emax - 86 - shift), both factors exact powers of two in
// range (x < 2^62, and the second's biased exponent emax + 41 - shift lies
// in [5, 254] for finite sums).  x itself goes through its two 32-bit halves
// (within one FP32 ulp).
__device__ __forceinline__ float from_fixed(uint64_t x, int emax, int shift)
{
    const float f = fmaf(__uint2float_rn(static_cast<uint32_t>(x >> 32)), 4294967296.0f,
                         __uint2float_rn(static_cast<uint32_t>(x)));
    const int e = min(emax + 41 - shift, 254);
    return (f * 0x1.0p-64f) * __int_as_float(e << 23);
}

// The first cumulative value that reaches u * total, u = uq * 2^-64: the
// smallest integer >= uq * tot / 2^64.
__device__ __forceinline__ uint64_t fixed_target(uint64_t uq, uint64_t tot)
{
    return __umul64hi(uq, tot) + ((uq * tot) != 0ull ? 1ull : 0ull);
}

// Event uniform in (0,1) as 64-bit fixed point: 47 random bits, (2A+1) 2^-48.
__device__ __forceinline__ uint64_t u01_fixed(uint32_t a, uint32_t b)
{
    const uint64_t A = ((static_cast<uint64_t>(a) << 15) | (b >> 17)) & ((1ull << 47) - 1);
    return ((A << 1) | 1ull) << 16;
}

// A replay uniform u in (0,1) as 64-bit fixed point (exact for u >= 2^-11).
__device__ __forceinline__ uint64_t u01_fixed_from_double(double u)
{
    return __double2ull_rz(u * 0x1.0p64);
}

// Exact n / T for 0 <= n < 2^22 from inv ~ 1/T (float reciprocal, one
// correction step), as in decode_pair below.
__device__ __forceinline__ int div_small(int n, int T, float inv)
{
    int q = __float2int_rz(__int2float_rn(n) * inv);
    const int r = n - q * T;
    if (r < 0) --q; else if (r >= T) ++q;
    return q;
}

// Row-aligned runs: thread g of a group of G walks the rows [row_bound(g),
// row_bound(g + 1)) of the pair enumeration (h source rows of T1 targets,
// then P rows of T2), the boundary nearest to pair g*A/G.  Every thread then
// starts each of its rows at column 0, so the threads of a group step
// through the same target column together.
__device__ __forceinline__ int row_bound(int g, int G, int A, int A1, int h, int P, int T1, int T2,
                                         float inv1, float inv2)
{
    if (g <= 0) return 0;
    if (g >= G) return h + P;
    const int k = static_cast<int>((static_cast<long long>(g) * A) / G);
    if (k < A1) return min(h, div_small(k + (T1 >> 1), T1, inv1));
    if (T2 <= 0) return h + P;
    return min(h + P, h + div_small(k - A1 + (T2 >> 1), T2, inv2));
}

// First pair of row r.
__device__ __forceinline__ int row_start(int r, int h, int A1, int T1, int T2)
{
    return r <= h ? r * T1 : A1 + (r - h) * T2;
}

// k -> (row, col) within the pair enumeration.  Float-reciprocal quotient
// with one correction step: with inv within 2^-22 (relative) of 1/T and
// k < 2^22 the estimate is off by less than one, so the result is exact (the
// engine limits S so that A(h) stays below 2^22).
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

// ---------------------------------------------------------------------------
// Pair-rate sources
// ---------------------------------------------------------------------------

// Table mode: records are {site, scaled energy}; (L, B) read from the table.
// kStaged: the launch's one table sits in shared memory (the pointer then
// derives from shared memory only, so its loads are shared-memory loads with
// 32-bit addresses); otherwise each chain reads its table from global memory.
// kUniform (staged only): every chain of the launch has the same kT, and the
// staged table holds (L, L + c B) with c = log2(e)/kT, so a pair's rate
// needs one add less; B itself is staged beside it for the energy updates.
// Every variant evaluates the same expression,
//     rate = 2^min(L, (L + c B) - (e_t - e_s)),  L + c B = fma(c, B, L),
// so a chain's result does not depend on which one runs it.
template <bool kStaged, bool kUniform = false>
struct TablePairs {
    using Rec = int2;
    static constexpr bool kSiteInRec = true;    // rec.x is the site id
    static constexpr bool kUniformTable = kUniform;
    static constexpr bool kPairedTgt = false;
    __device__ __forceinline__ static int site(Rec r) { return r.x; }
    const float2 *tab;
    const float *coul;   // kUniform: B of each pair
    int S;
    __device__ __forceinline__ void init(const kmc_batch &B, int t_id, int S_, const float2 *shared_tab)
    {
        if (kStaged)
            tab = shared_tab;
        else
            tab = reinterpret_cast<const float2 *>(B.tab_LB + B.tab_off[t_id]);
        S = S_;
        coul = kUniform ? reinterpret_cast<const float *>(shared_tab + S_ * S_) : nullptr;
    }
    __device__ __forceinline__ Rec rec(int site, float e) const { return make_int2(site, __float_as_int(e)); }
    __device__ __forceinline__ float rate(Rec s, Rec t, bool /*acc*/, float cs) const
    {
        const float2 lb = tab[s.x * S + t.x];
        const float d = __int_as_float(t.y) - __int_as_float(s.y);
        const float lcb = kUniform ? lb.y : fmaf(cs, lb.y, lb.x);
        return ex2_approx(fminf(lb.x, lcb - d));
    }
    // the table carries the Coulomb term: no per-pair coefficient
    __device__ __forceinline__ float rate_k(Rec s, Rec t, float /*k*/, float cs) const { return rate(s, t, false, cs); }
    __device__ __forceinline__ static float coulomb_coef(float) { return 0.0f; }
    // Coulomb term I_0 R / d_jk between acceptors j, k (0 on the diagonal).
    __device__ __forceinline__ float coulomb(int j, int k) const
    {
        return kUniform ? coul[j * S + k] : tab[j * S + k].y;
    }
};

// Positions mode: records are {x, y, z, scaled energy}; d from coordinates.
struct PositionPairs {
    using Rec = float4;
    static constexpr bool kSiteInRec = false;   // site ids kept beside the records
    static constexpr bool kUniformTable = false;
    static constexpr bool kPairedTgt = false;
    __device__ __forceinline__ static int site(Rec) { return -1; }
    const float4 *pos;
    float kL, L0, IR;
    __device__ __forceinline__ void init(const kmc_batch &B, int t_id, int /*S*/, const float2 *)
    {
        pos = reinterpret_cast<const float4 *>(B.tab_pos + B.tab_pos_off[t_id]);
        const float4 c = reinterpret_cast<const float4 *>(B.tab_coef)[t_id];
        kL = c.x;    // -2 log2(e) / ab
        L0 = c.y;    // log2(nu * nu)
        IR = c.z;    // I_0 R
    }
    __device__ __forceinline__ Rec rec(int site, float e) const
    {
        const float4 p = __ldg(&pos[site]);
        return make_float4(p.x, p.y, p.z, e);
    }
    __device__ __forceinline__ float rate(Rec s, Rec t, bool acc, float cs) const
    {
        const float dx = t.x - s.x, dy = t.y - s.y, dz = t.z - s.z;
        const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        const float rs = rsqrt_approx(d2);
        const float L = fmaf(kL, d2 * rs, L0);
        float x = t.w - s.w;
        if (acc) x = fmaf(-cs * IR, rs, x);
        x = fmaxf(x, 0.0f);
        return ex2_approx(L - x);
    }
    // The same rate with the Coulomb coefficient given: k = coulomb_coef(cs)
    // for a pair of acceptors, 0 otherwise (fma(0, rs, x) is x exactly, so
    // both forms give the same bits).
    __device__ __forceinline__ float rate_k(Rec s, Rec t, float k, float /*cs*/) const
    {
        const float dx = t.x - s.x, dy = t.y - s.y, dz = t.z - s.z;
        const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        const float rs = rsqrt_approx(d2);
        const float L = fmaf(kL, d2 * rs, L0);
        const float x = fmaxf(fmaf(k, rs, t.w - s.w), 0.0f);
        return ex2_approx(L - x);
    }
    __device__ __forceinline__ float coulomb_coef(float cs) const { return -cs * IR; }
    __device__ __forceinline__ float coulomb(int j, int k) const
    {
        if (j == k) return 0.0f;
        const float4 a = __ldg(&pos[j]), b = __ldg(&pos[k]);
        const float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
        return IR * rsqrt_approx(fmaf(dx, dx, fmaf(dy, dy, dz * dz)));
    }
};

// Positions mode for block groups.  The target list is stored in pairs,
// component by component ({x0, x1, y0, y1, z0, z1, w0, w1} for targets 2m
// and 2m + 1), so two targets of a row load as two 16-byte words whose
// halves are packed FP32 pairs, and the row-aligned walk evaluates both
// pairs with the packed FP32x2 add / mul / fma (one instruction for two
// pairs).  Each lane performs the operations of rate_k in the same order
// with the same rounding: the rates are bit-identical to the scalar walk's.
struct PairedPositionPairs : PositionPairs {
    static constexpr bool kPairedTgt = true;
    // targets (xy, zw) = {x0, x1, y0, y1}, {z0, z1, w0, w1} from a source
    // whose negated record is ns, with Coulomb coefficient k (rate_k)
    __device__ __forceinline__ void rate2(const float4 &xy, const float4 &zw, const float4 &ns, float k,
                                          float &ra, float &rb) const
    {
        const float2 dx = __fadd2_rn(make_float2(xy.x, xy.y), make_float2(ns.x, ns.x));
        const float2 dy = __fadd2_rn(make_float2(xy.z, xy.w), make_float2(ns.y, ns.y));
        const float2 dz = __fadd2_rn(make_float2(zw.x, zw.y), make_float2(ns.z, ns.z));
        const float2 d2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __fmul2_rn(dz, dz)));
        const float2 rs = make_float2(rsqrt_approx(d2.x), rsqrt_approx(d2.y));
        const float2 L = __ffma2_rn(make_float2(kL, kL), __fmul2_rn(d2, rs), make_float2(L0, L0));
        const float2 x = __ffma2_rn(make_float2(k, k), rs, __fadd2_rn(make_float2(zw.z, zw.w), make_float2(ns.w, ns.w)));
        // L - max(x, 0) as L + min(-x, -0): the same value (signed zeros
        // included, both give L when x <= 0)
        const float2 y = __fadd2_rn(L, make_float2(fminf(-x.x, -0.0f), fminf(-x.y, -0.0f)));
        ra = ex2_approx(y.x);
        rb = ex2_approx(y.y);
    }
};

// Target records: a plain array, or (kPairedTgt) pairs stored component by
// component; col is the target's position in the list.
template <typename Pairs>
__device__ __forceinline__ typename Pairs::Rec tgt_load(const typename Pairs::Rec *t, int col)
{
    if constexpr (Pairs::kPairedTgt) {
        const float *f = reinterpret_cast<const float *>(t) + (col >> 1) * 8 + (col & 1);
        return make_float4(f[0], f[2], f[4], f[6]);
    } else {
        return t[col];
    }
}
template <typename Pairs>
__device__ __forceinline__ void tgt_store(typename Pairs::Rec *t, int col, const typename Pairs::Rec &r)
{
    if constexpr (Pairs::kPairedTgt) {
        float *f = reinterpret_cast<float *>(t) + (col >> 1) * 8 + (col & 1);
        f[0] = r.x;
        f[2] = r.y;
        f[4] = r.z;
        f[6] = r.w;
    } else {
        t[col] = r;
    }
}

// ---------------------------------------------------------------------------
// Thread groups: a G-lane slice of a warp, or a whole block
// ---------------------------------------------------------------------------

template <int G>
struct WarpGroup {
    static constexpr int kSize = G;
    int g;            // rank in the group
    int sub;          // group index within the warp
    unsigned mask;
    __device__ __forceinline__ void init()
    {
        const int lane = threadIdx.x & 31;
        sub = lane / G;
        g = lane % G;
        mask = (G == 32 ? 0xffffffffu : ((1u << G) - 1u)) << (sub * G);
    }
    __device__ __forceinline__ void sync() const { __syncwarp(mask); }
    __device__ __forceinline__ float scanf(float v, float &tot) const
    {
        float x = v;
#pragma unroll
        for (int d = 1; d < G; d <<= 1) {
            const float o = __shfl_up_sync(mask, x, d, G);
            if (g >= d) x += o;
        }
        tot = __shfl_sync(mask, x, G - 1, G);
        return x;
    }
    // lowest / highest rank with p true, or -1
    __device__ __forceinline__ int first(bool p) const
    {
        const unsigned low = (G == 32) ? 0xffffffffu : ((1u << G) - 1u);
        const unsigned b = (__ballot_sync(mask, p) >> (sub * G)) & low;
        return b ? __ffs(b) - 1 : -1;
    }
    __device__ __forceinline__ int last(bool p) const
    {
        const unsigned low = (G == 32) ? 0xffffffffu : ((1u << G) - 1u);
        const unsigned b = (__ballot_sync(mask, p) >> (sub * G)) & low;
        return b ? 31 - __clz(b) : -1;
    }
    template <typename V>
    __device__ __forceinline__ V bcast(V v, int src) const { return __shfl_sync(mask, v, src, G); }
    __device__ __forceinline__ uint32_t max_u32(uint32_t v) const { return __reduce_max_sync(mask, v); }
    __device__ __forceinline__ float sumf(float v) const
    {
#pragma unroll
        for (int d = G / 2; d >= 1; d >>= 1) v += __shfl_xor_sync(mask, v, d, G);
        return v;
    }
#ifdef KMC_DEBUG_CHECKS
    // FP64 inclusive scan (debug builds: the cross-check of the selection)
    __device__ double scan_f64(double v, double &excl, double &tot) const
    {
        double x = v;
        for (int d = 1; d < G; d <<= 1) {
            const double o = __shfl_up_sync(mask, x, d, G);
            if (g >= d) x += o;
        }
        const double e = __shfl_up_sync(mask, x, 1, G);
        excl = g == 0 ? 0.0 : e;
        tot = __shfl_sync(mask, x, G - 1, G);
        return x;
    }
#endif
    // inclusive integer scan; sets the exclusive value and the total
    __device__ __forceinline__ uint64_t scan_u64(uint64_t v, uint64_t &excl, uint64_t &tot) const
    {
        uint64_t x = v;
#pragma unroll
        for (int d = 1; d < G; d <<= 1) {
            const uint64_t o = __shfl_up_sync(mask, x, d, G);
            if (g >= d) x += o;
        }
        excl = x - v;
        tot = __shfl_sync(mask, x, G - 1, G);
        return x;
    }
};

// Block-wide group; its scratch lives in static shared memory.
template <int T>
struct BlockGroup {
    static constexpr int kSize = T;
    static constexpr int kWarps = T / 32;
    int g;
    double *sd;   // [kWarps + 2]
    int *si;      // [2]
    __device__ __forceinline__ void init() { g = threadIdx.x; }
    __device__ __forceinline__ void sync() const { __syncthreads(); }
    __device__ float scanf(float v, float &tot) const
    {
        const int lane = g & 31, w = g >> 5;
        float x = v;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const float o = __shfl_up_sync(0xffffffffu, x, d);
            if (lane >= d) x += o;
        }
        float *sf = reinterpret_cast<float *>(sd);
        if (lane == 31) sf[w] = x;
        __syncthreads();
        if (w == 0) {
            float y = lane < kWarps ? sf[lane] : 0.0f;
#pragma unroll
            for (int d = 1; d < kWarps; d <<= 1) {
                const float o = __shfl_up_sync(0xffffffffu, y, d);
                if (lane >= d) y += o;
            }
            if (lane < kWarps) sf[lane] = y;
        }
        __syncthreads();
        const float base = w > 0 ? sf[w - 1] : 0.0f;
        tot = sf[kWarps - 1];
        __syncthreads();
        return x + base;
    }
    __device__ int first(bool p) const
    {
        if (g == 0) si[0] = 0x7fffffff;
        __syncthreads();
        if (p) atomicMin(&si[0], g);
        __syncthreads();
        const int r = si[0];
        __syncthreads();
        return r == 0x7fffffff ? -1 : r;
    }
    __device__ int last(bool p) const
    {
        if (g == 0) si[1] = -1;
        __syncthreads();
        if (p) atomicMax(&si[1], g);
        __syncthreads();
        const int r = si[1];
        __syncthreads();
        return r;
    }
#ifdef KMC_DEBUG_CHECKS
    __device__ double scan_f64(double v, double &excl, double &tot) const
    {
        const int lane = g & 31, w = g >> 5;
        double x = v;
        for (int d = 1; d < 32; d <<= 1) {
            const double o = __shfl_up_sync(0xffffffffu, x, d);
            if (lane >= d) x += o;
        }
        if (lane == 31) sd[w] = x;
        __syncthreads();
        if (w == 0) {
            double y = lane < kWarps ? sd[lane] : 0.0;
            for (int d = 1; d < kWarps; d <<= 1) {
                const double o = __shfl_up_sync(0xffffffffu, y, d);
                if (lane >= d) y += o;
            }
            if (lane < kWarps) sd[lane] = y;
        }
        __syncthreads();
        const double base = w > 0 ? sd[w - 1] : 0.0;
        tot = sd[kWarps - 1];
        __syncthreads();
        x += base;
        const double prev = __shfl_up_sync(0xffffffffu, x, 1);
        excl = lane > 0 ? prev : base;
        return x;
    }
#endif
    __device__ float sumf(float v) const
    {
        float tot;
        scanf(v, tot);
        return tot;
    }
    __device__ uint32_t max_u32(uint32_t v) const
    {
        const uint32_t w = __reduce_max_sync(0xffffffffu, v);
        uint32_t *s = reinterpret_cast<uint32_t *>(sd);   // kWarps slots
        if ((g & 31) == 0) s[g >> 5] = w;
        __syncthreads();
        uint32_t m = s[0];
#pragma unroll
        for (int k = 1; k < kWarps; ++k) m = max(m, s[k]);
        __syncthreads();
        return m;
    }
    __device__ uint64_t scan_u64(uint64_t v, uint64_t &excl, uint64_t &tot) const
    {
        const int lane = g & 31, w = g >> 5;
        uint64_t x = v;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint64_t o = __shfl_up_sync(0xffffffffu, x, d);
            if (lane >= d) x += o;
        }
        uint64_t *s = reinterpret_cast<uint64_t *>(sd);   // kWarps slots
        if (lane == 31) s[w] = x;
        __syncthreads();
        if (w == 0) {
            uint64_t y = lane < kWarps ? s[lane] : 0ull;
#pragma unroll
            for (int d = 1; d < kWarps; d <<= 1) {
                const uint64_t o = __shfl_up_sync(0xffffffffu, y, d);
                if (lane >= d) y += o;
            }
            if (lane < kWarps) s[lane] = y;
        }
        __syncthreads();
        const uint64_t base = w > 0 ? s[w - 1] : 0ull;
        tot = s[kWarps - 1];
        __syncthreads();
        x += base;
        excl = x - v;
        return x;
    }
    template <typename V>
    __device__ V bcast(V v, int src) const
    {
        static_assert(sizeof(V) <= sizeof(double), "bcast slot holds one double");
        V *slot = reinterpret_cast<V *>(sd + kWarps);
        if (g == src) *slot = v;
        __syncthreads();
        const V r = *slot;
        __syncthreads();
        return r;
    }
};

// ---------------------------------------------------------------------------
// Per-chain shared memory
// ---------------------------------------------------------------------------


template <typename Rec>
struct ChainSmem {
    Rec *src;        // [S+2] source records
    Rec *tgt;        // [S+2] target records (paired layout: tgt_load / tgt_store)
    int *src_id;     // [S+1] site ids of the sources
    int *tgt_id;     // [S+1] site ids of the targets
    float *E;        // [S]   site energies (acceptors), high part
    float *Elo;      // [S]   their low parts: E + Elo carries the energy to ~2^-47
    uint32_t *occw;  // [W]   occupancy bits
    int *eo;         // [kMaxElectrodes] electrode counters of this launch
    float *rates;    // [rate_words] this hop's pair rates, or nullptr (recompute)
    int rate_words;  // words of `rates`
#ifdef KMC_DEBUG_CHECKS
    int rate_cap;    // words of `rates`
#endif
};

template <typename Rec>
__host__ __device__ __forceinline__ int chain_list_words(int S)
{
    const int W = (S + 31) / 32;
    const int rw = static_cast<int>(sizeof(Rec) / 4);
    const int words = 2 * rw * (S + 2) + 2 * (S + 1) + 2 * S + W + kMaxElectrodes;
    return (words + 3) & ~3;
}

#ifndef KMC_RATE_PAD
#define KMC_RATE_PAD 1
#endif
// Row stride of the stored running sums: element i of thread g of a G-thread
// group sits at i*(G + 1) + g.  The threads store row i together (one
// conflict-free wavefront), and the search, where thread g reads element g of
// one thread's column, hits G distinct banks (with a stride of G it would hit
// 32/gcd(G, 32) banks: 8-way conflicts for G = 16).
template <int G>
struct RateStride {
    static constexpr int kValue = G + KMC_RATE_PAD;
};

// Words to keep every pair rate of one hop: A(h) <= S^2/3 for any split of
// S sites into acceptors and electrodes; the transposed layout (element i of
// thread g at i*(G + 1) + g, i < M) reaches (G + 1)*M <= A + A/G + 2G + 2
// with M <= A/G + 2 (rounded up to odd).
__host__ __device__ __forceinline__ int rate_buffer_words(int S, int G)
{
    const int A = (S * S) / 3 + 1;
    return ((A + A / G + 2 * G + 2) + 3) & ~3;
}

template <typename Rec>
__device__ __forceinline__ ChainSmem<Rec> carve(uint32_t *base, int S, int rate_words)
{
    ChainSmem<Rec> c;
    c.src = reinterpret_cast<Rec *>(base);
    c.tgt = c.src + (S + 2);
    c.src_id = reinterpret_cast<int *>(c.tgt + (S + 2));
    c.tgt_id = c.src_id + (S + 1);
    c.E = reinterpret_cast<float *>(c.tgt_id + (S + 1));
    c.Elo = c.E + S;
    c.occw = reinterpret_cast<uint32_t *>(c.Elo + S);
    c.eo = reinterpret_cast<int *>(c.occw + (S + 31) / 32);
    c.rates = rate_words > 0 ? reinterpret_cast<float *>(base + chain_list_words<Rec>(S)) : nullptr;
    c.rate_words = rate_words > 0 ? rate_words : 0;
#ifdef KMC_DEBUG_CHECKS
    c.rate_cap = rate_words;
#endif
    return c;
}

// ---------------------------------------------------------------------------
// The hop loop of one chain, run by one group
// ---------------------------------------------------------------------------

template <typename Grp, typename Pairs>
__device__ void run_chain(const kmc_batch &B, const Grp &grp, ChainSmem<typename Pairs::Rec> sm,
                          int c, const float2 *shared_tab)
{
    constexpr int G = Grp::kSize;
    constexpr int RS = RateStride<G>::kValue;
    using Rec = typename Pairs::Rec;
    const int g = grp.g;
    const int t_id = B.chain_tab[c];
    const int N = B.tab_N[t_id];
    const int P = B.tab_P[t_id];
    const int S = N + P;
    if (P > kMaxElectrodes || S > B.max_sites || N < 0) {
        if (g == 0) B.status[c] = KMC_ERR_INVALID;
        return;
    }
    Pairs pairs;
    pairs.init(B, t_id, S, shared_tab);
    const int64_t so = B.chain_site_off[c];
    const int64_t eoff = B.chain_el_off[c];
    const float *Ec = B.E_constant + so;
    const float *Vel = B.el_energy + eoff;
    uint8_t *occ_g = B.occupation + so;
    const float cs = kLog2e / B.chain_kT[c];
    if (Pairs::kUniformTable && !(B.chain_kT[c] == B.uniform_kT)) {
        // the staged table was scaled for another temperature
        if (g == 0) B.status[c] = KMC_ERR_INVALID;
        return;
    }
    const int64_t hops_done0 = B.hops_done[c];
    int64_t todo = B.hops_total[c] - hops_done0;
    if (todo > B.max_hops_per_launch) todo = B.max_hops_per_launch;
    const uint64_t stream = B.stream[c];
    const uint32_t k0 = static_cast<uint32_t>(B.seed), k1 = static_cast<uint32_t>(B.seed >> 32);
    const int record = B.record;
    const int reanchor = B.reanchor > 0 ? B.reanchor : 1024;
    const int W = (N + 31) / 32;

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
    grp.sync();
    int h = 0;
    for (int w = 0; w < W; ++w) h += __popc(sm.occw[w]);

    double t = B.time[c];    // the clock: FP64 (one add per hop, off the critical path)
    int64_t hop = hops_done0;
#ifdef KMC_DEBUG_CHECKS
    int dbg_bad = 0;
#endif
    const uint64_t t_launch = B.time_budget_ns > 0 ? globaltimer_ns() : 0;
    const int64_t hop_end = hops_done0 + (todo > 0 ? todo : 0);
    int status = KMC_OK;
    unsigned long long npairs = 0;
    const double *replay = B.replay ? B.replay + B.replay_off[c] : nullptr;
    double *occ_time = record ? B.occ_time + so : nullptr;
    double *occ_since = record ? B.occ_since + so : nullptr;
    int32_t *traffic = record ? B.traffic + B.chain_pair_off[c] : nullptr;
    if (record)
        for (int j = g; j < N; j += G) occ_since[j] = t;

    // Energies from scratch (E_j = Ec_j - sum_{k empty} B_jk) and the ordered
    // lists built from them.  Run at the launch start and at every absolute
    // hop index that is a multiple of `reanchor`, so a run split into
    // launches anchors at the same hops.
    // With `drift`, the energies the incremental updates carried since the
    // last anchor are compared with the recomputed ones first, and the
    // largest difference (in units of kT) is kept per chain.
    float drift_max = 0.0f;
    // Compensated energies (TwoSum per increment) in block groups, where
    // networks are large and hundreds of terms per hop would otherwise let
    // the FP32 energies drift by up to 0.02 kT between re-anchors (measured
    // on N=1000 networks); warp slices run small networks whose drift stays
    // near 1e-3 kT and keep one add per increment (the compensation cost
    // 2.5 % of the N=30 ensemble's throughput).
    constexpr bool kComp = G >= 64;
    auto eadd = [](float &hi, float &lo, float c) {
        if (kComp) comp_add(hi, lo, c);
        else hi += c;
    };
    // The record of electrode g (thread g < P), the same every hop of the
    // launch: the rebuilds after a hop copy it instead of reading the
    // electrode's energy from global memory again.
    Rec el_rec{};
    auto anchor_and_build = [&](bool drift) {
        for (int j = g; j < N; j += G) {
            // E_j = Ec_j - sum_{k empty} B_jk, summed with compensation
            float hi = Ec[j], lo = 0.0f;
            for (int k = 0; k < N; ++k)
                if (!((sm.occw[k >> 5] >> (k & 31)) & 1u)) eadd(hi, lo, -pairs.coulomb(j, k));
            if (drift) drift_max = fmaxf(drift_max, fabsf((hi - sm.E[j]) + (lo - (kComp ? sm.Elo[j] : 0.0f))));
            sm.E[j] = hi;
            if (kComp) sm.Elo[j] = lo;
        }
        const int z = N - h;
        int wcur = 0, cum = 0;
        for (int j = g; j < N; j += G) {
            const int w = j >> 5;
            while (wcur < w) { cum += __popc(sm.occw[wcur]); ++wcur; }
            const uint32_t word = sm.occw[w];
            const int below = cum + __popc(word & ((1u << (j & 31)) - 1u));
            const Rec r = pairs.rec(j, cs * (kComp ? sm.E[j] + sm.Elo[j] : sm.E[j]));
            if ((word >> (j & 31)) & 1u) {
                sm.src[below] = r;
                if (!Pairs::kSiteInRec) sm.src_id[below] = j;
            } else {
                tgt_store<Pairs>(sm.tgt, j - below, r);
                if (!Pairs::kSiteInRec) sm.tgt_id[j - below] = j;
            }
        }
        for (int e = g; e < P; e += G) {
            const Rec r = pairs.rec(N + e, cs * Vel[e]);
            if (e == g) el_rec = r;   // kept for the list rebuilds of later hops
            sm.src[h + e] = r;
            tgt_store<Pairs>(sm.tgt, z + e, r);
            if (!Pairs::kSiteInRec) {
                sm.src_id[h + e] = N + e;
                sm.tgt_id[z + e] = N + e;
            }
        }
        grp.sync();
    };
    anchor_and_build(false);
    int until_anchor = reanchor - static_cast<int>(hop % reanchor);

    // Thread g holds the two uniforms of hop rbase + (g mod 32), already
    // mapped: the clock's Exp(1) variate and the event uniform.
    float rnd_e1 = 0.0f;
    uint64_t rnd_u = 0;
    int64_t rbase = INT64_MIN / 2;
    constexpr int RW = G < 32 ? G : 32;   // hops per refill

#ifdef KMC_SECTION_CLOCKS
    uint32_t sec_cycles[kSections] = {};
    uint32_t sec_last = static_cast<uint32_t>(clock());
#endif
    while (hop < hop_end) {
        if ((hop & 1023) == 0 && (B.cancel || (B.time_budget_ns > 0 && hop != hops_done0))) {
            // the host's cancel word, then the launch's wall-clock budget
            int stop = 0;
            if (g == 0) {
                if (B.cancel && *B.cancel) stop = KMC_ERR_CANCELLED;
                else if (B.time_budget_ns > 0 && hop != hops_done0 &&
                         static_cast<int64_t>(globaltimer_ns() - t_launch) > B.time_budget_ns)
                    stop = KMC_ERR_TIMEOUT;
            }
            stop = grp.bcast(stop, 0);
            if (stop) { status = stop; break; }
        }
        if (until_anchor == 0) {
            grp.sync();           // bit updates of the last hop are visible
            anchor_and_build(B.energy_drift != nullptr);
            until_anchor = reanchor;
        }
        --until_anchor;
        KMC_SECTION(0);
        // ---- pair phase ----
        const int z = N - h;
        const int T1 = z + P, T2 = z;
        const int A1 = h * T1;
        const int A = A1 + P * T2;
        if (A <= 0) { status = KMC_ERR_NONFINITE; break; }
        const float inv1 = T1 > 0 ? rcp_approx(static_cast<float>(T1)) : 0.0f;
        const float inv2 = T2 > 0 ? rcp_approx(static_cast<float>(T2)) : 0.0f;
        // Two ways to split the A pairs into G contiguous runs.  Balanced:
        // thread g takes [g*M, g*M + M) whatever the rows, and keeps track of
        // row changes pair by pair.  Row-aligned: thread g takes whole rows
        // [row_bound(g), row_bound(g + 1)), the boundaries nearest to pair
        // g*A/G, so every thread starts each row at column 0: the threads of a
        // group read the same target record at the same time (one broadcast
        // load) and need no per-pair row bookkeeping, at the price of runs up
        // to one row longer than A/G and a loop set-up per row.  Measured on
        // GB300: +47 % on N=1000 networks (rows of ~108 targets, block groups
        // of 256 threads), -26 % on the N=30 ensemble (rows of 11, warp
        // slices), and even compiled in but not taken it cost the warp-slice
        // kernels 3 %: block groups take row-aligned runs for rows of at
        // least 32 targets and runs of at least 1.5 rows; warp slices are
        // compiled with balanced runs only.
#ifdef KMC_FORCE_BALANCED_RUNS
        constexpr bool kAlignedRuns = false;   // measurement builds: the balanced split only
#else
        constexpr bool kAlignedRuns = G >= 64;
#endif
        const bool aligned = kAlignedRuns && T1 >= 32 && A >= ((3 * G * T1) >> 1);
        // Balanced run length.  Block groups round it up to an odd number:
        // thread g's run starts M records after thread g-1's, and with long
        // rows an odd stride puts the threads' record loads in distinct banks.
        const int M = ((A + G - 1) / G) | (G >= 64 ? 1 : 0);
        int run_b, run_e, r0 = 0, r1 = 0;
        if (aligned) {
            r0 = row_bound(g, G, A, A1, h, P, T1, T2, inv1, inv2);
            r1 = row_bound(g + 1, G, A, A1, h, P, T1, T2, inv1, inv2);
            run_b = row_start(r0, h, A1, T1, T2);
            run_e = row_start(r1, h, A1, T1, T2);
        } else {
            run_b = min(g * M, A);
            run_e = min(run_b + M, A);
        }
        // the running sum after every pair is kept (transposed: element i of
        // thread g at i*RS + g) when every run of the group fits the buffer
        const bool stored = sm.rates != nullptr &&
                            (aligned ? static_cast<int>(grp.max_u32(static_cast<uint32_t>(run_e - run_b))) * RS
                                     : M * RS) <= sm.rate_words;
        float lsum = 0.0f;
        float *rp = stored ? sm.rates + g : nullptr;
        // The pair walks, compiled once storing the running sums and once not
        // (no per-pair test of the choice).
        auto walk_aligned = [&](auto store) {
            constexpr bool kStore = decltype(store)::value;
            const float kacc = pairs.coulomb_coef(cs);
            for (int row = r0; row < r1; ++row) {
                KMC_DCHECK(row >= 0 && row < h + P);
                const Rec sr = sm.src[row];
                const bool sa = row < h;
                const int Tc = sa ? T1 : T2;
                // columns [0, z) are acceptors (with the Coulomb term when the
                // source is one too), [z, Tc) electrodes
                for (int seg = 0; seg < 2; ++seg) {
                    const int c1 = seg ? Tc : z;
                    const float k = (seg == 0 && sa) ? kacc : 0.0f;
                    int col = seg ? z : 0;
                    if constexpr (Pairs::kPairedTgt) {
                        // an odd first column alone, then whole target pairs:
                        // two 16-byte loads and packed arithmetic per two pairs
                        if ((col & 1) && col < c1) {
                            lsum += pairs.rate_k(sr, tgt_load<Pairs>(sm.tgt, col), k, cs);
                            if constexpr (kStore) { rp[0] = lsum; rp += RS; }
                            ++col;
                        }
                        const float4 ns = make_float4(-sr.x, -sr.y, -sr.z, -sr.w);
                        const float *tf = reinterpret_cast<const float *>(sm.tgt);
#pragma unroll kPairUnroll
                        for (; col + 1 < c1; col += 2) {
                            const float4 xy = *reinterpret_cast<const float4 *>(tf + col * 4);
                            const float4 zw = *reinterpret_cast<const float4 *>(tf + col * 4 + 4);
                            float ra, rb;
                            pairs.rate2(xy, zw, ns, k, ra, rb);
                            lsum += ra;
                            if constexpr (kStore) rp[0] = lsum;
                            lsum += rb;
                            if constexpr (kStore) { rp[RS] = lsum; rp += 2 * RS; }
                        }
                    } else {
#pragma unroll kPairUnroll
                        for (; col + 1 < c1; col += 2) {
                            const float ra = pairs.rate_k(sr, tgt_load<Pairs>(sm.tgt, col), k, cs);
                            const float rb = pairs.rate_k(sr, tgt_load<Pairs>(sm.tgt, col + 1), k, cs);
                            lsum += ra;
                            if constexpr (kStore) rp[0] = lsum;
                            lsum += rb;
                            if constexpr (kStore) { rp[RS] = lsum; rp += 2 * RS; }
                        }
                    }
                    if (col < c1) {
                        lsum += pairs.rate_k(sr, tgt_load<Pairs>(sm.tgt, col), k, cs);
                        if constexpr (kStore) { rp[0] = lsum; rp += RS; }
                    }
                }
            }
        };
        auto walk_balanced = [&](auto store) {
            constexpr bool kStore = decltype(store)::value;
            // The thread walks its run in row-major order, two pairs per step
            // (two independent load -> rate chains; a row change is a select
            // plus a predicated reload, not a branch).
            const int kb = run_b, ke = run_e;
            int row, col;
            decode_pair(kb, h, A1, T1, T2, inv1, inv2, row, col);
            KMC_DCHECK(ke <= A && row >= 0 && row < h + P && col >= 0 && col < (row < h ? T1 : T2));
            bool sa = row < h;
            int Tc = sa ? T1 : T2;
            Rec sr = sm.src[row];
            int k = kb;
#pragma unroll kPairUnroll
            for (; k + 1 < ke; k += 2) {
                // second pair of the step
                const bool wa = (col + 1 == Tc);
                const int colb = wa ? 0 : col + 1;
                const int rowb = row + (wa ? 1 : 0);
                Rec srb = sr;
                if (wa) srb = sm.src[rowb];        // reload only on a row change
                const bool sab = rowb < h;
                const int Tcb = sab ? T1 : T2;
                const float ra = pairs.rate(sr, tgt_load<Pairs>(sm.tgt, col), sa && col < z, cs);
                const float rb = pairs.rate(srb, tgt_load<Pairs>(sm.tgt, colb), sab && colb < z, cs);
                lsum += ra;
                if constexpr (kStore) rp[0] = lsum;
                lsum += rb;
                if constexpr (kStore) { rp[RS] = lsum; rp += 2 * RS; }
                // advance past the second pair
                const bool wb = (colb + 1 == Tcb);
                col = wb ? 0 : colb + 1;
                row = rowb + (wb ? 1 : 0);
                sr = srb;
                if (wb) sr = sm.src[row];
                sa = row < h;
                Tc = sa ? T1 : T2;
            }
            if (k < ke) {
                lsum += pairs.rate(sr, tgt_load<Pairs>(sm.tgt, col), sa && col < z, cs);
                if constexpr (kStore) rp[0] = lsum;
            }
        };
        if (aligned) {
            if (rp) walk_aligned(BoolC<true>{});
            else walk_aligned(BoolC<false>{});
        } else if (run_b < run_e) {
            if (rp) walk_balanced(BoolC<true>{});
            else walk_balanced(BoolC<false>{});
        }
        // the run [b, e) of thread l of the group
        auto run_of = [&](int l, int &b, int &e) {
            if (aligned) {
                b = row_start(row_bound(l, G, A, A1, h, P, T1, T2, inv1, inv2), h, A1, T1, T2);
                e = row_start(row_bound(l + 1, G, A, A1, h, P, T1, T2, inv1, inv2), h, A1, T1, T2);
            } else {
                b = min(l * M, A);
                e = min(b + M, A);
            }
        };
        npairs += static_cast<unsigned long long>(A);
        KMC_SECTION(1);
        // ---- uniforms for this hop ----
        uint64_t u_ev;
        float e1;
        if (replay) {
            e1 = -log1pf(-static_cast<float>(replay[2 * hop]));
            u_ev = u01_fixed_from_double(replay[2 * hop + 1]);
        } else {
            if (hop - rbase >= RW) {
                rbase = hop;
                const uint64_t ctr = static_cast<uint64_t>(hop + (g & 31));
                const u32x4 w = philox4x32_10(u32x4{static_cast<uint32_t>(ctr), static_cast<uint32_t>(ctr >> 32),
                                                    static_cast<uint32_t>(stream),
                                                    static_cast<uint32_t>(stream >> 32)},
                                              k0, k1);
                // Exp(1) clock variate: logf (within an ulp; once per G hops
                // per thread) of a 32-bit uniform
                rnd_e1 = -logf(u01_tail32(w.x));
                rnd_u = u01_fixed(w.y, w.z);
            }
            const int ri = static_cast<int>(hop - rbase);
            e1 = grp.bcast(rnd_e1, ri);
            u_ev = grp.bcast(rnd_u, ri);
        }
        if (stored) grp.sync();   // stored rates visible to the whole group
        KMC_SECTION(2);
        // ---- exact fixed-point scan of the per-thread sums ----
        // scale: the largest per-thread sum (positive FP32 values order as
        // their bit patterns; NaN and infinity sit above every finite value)
        const uint32_t mx = grp.max_u32(__float_as_uint(lsum));
        if (mx == 0u || mx >= 0x7f800000u) { status = KMC_ERR_NONFINITE; break; }
        constexpr int kShift = FixShift<G>::kShift;
        const int emax = static_cast<int>(mx >> 23);
        uint64_t excl, tot;
        const uint64_t incl = grp.scan_u64(to_fixed(lsum, emax, kShift), excl, tot);
        const float totf = from_fixed(tot, emax, kShift);
        if (!(totf <= 3.0e38f)) { status = KMC_ERR_NONFINITE; break; }
        // the event is the first pair whose cumulative rate reaches u*total:
        // thread L's run holds it (tot >= target, so some thread qualifies)
        const uint64_t target = fixed_target(u_ev, tot);
        int L = grp.first(incl >= target);
        if (L < 0) L = grp.last(run_e > run_b);
        // what remains of u*total beyond the runs before L, back in FP32
        float rem = grp.bcast(from_fixed(target - excl, emax, kShift), L);
        KMC_SECTION(3);
        // ---- find the event inside thread L's run ----
        int chosen = -1, last_pos = -1;
        if (!(rem > 0.0f)) rem = 1.0e-38f;   // first pair with a positive rate
        int kbL, keL;
        run_of(L, kbL, keL);
        if (stored) {
            // Thread L kept its running sums: the event is the first pair whose
            // sum reaches rem.  Each thread of the group searches one block of
            // them; the lowest block with a hit wins.
            const int len = keL - kbL;
            // Thread g tests elements g, g + G, ... of thread L's run, a chunk
            // of G elements per round with both rounds' loads issued first;
            // the running sums do not decrease, so the lowest element of the
            // first chunk with a hit is the event.
            int idx = -1;
            for (int i0 = 0; i0 < len && idx < 0; i0 += 2 * G) {
                const int ia = i0 + g, ib = i0 + G + g;
                const float va = ia < len ? sm.rates[ia * RS + L] : -1.0f;
                const float vb = ib < len ? sm.rates[ib * RS + L] : -1.0f;
                const int ha = grp.first(va >= rem);
                const int hb = grp.first(vb >= rem);
                if (ha >= 0) idx = i0 + ha;
                else if (hb >= 0) idx = i0 + G + hb;
            }
            if (idx >= 0) {
                chosen = kbL + idx;
            } else if (len > 0) {
                // rem rounded above the run's total: the run's last pair
                // with a positive rate
                int lp = -1;
                for (int i = g; i < len; i += G)
                    if (sm.rates[i * RS + L] > (i > 0 ? sm.rates[(i - 1) * RS + L] : 0.0f)) lp = i;
                const int ll = static_cast<int>(grp.max_u32(static_cast<uint32_t>(lp + 1))) - 1;
                if (ll >= 0) chosen = kbL + ll;
            }
        } else {
            const int kb = kbL;
            const int len = keL - kbL;
            for (int i0 = 0; i0 < len; i0 += G) {
                const int i = i0 + g;
                float r = 0.0f;
                if (i < len) {
                    int row, col;
                    decode_pair(kb + i, h, A1, T1, T2, inv1, inv2, row, col);
                    r = pairs.rate(sm.src[row], tgt_load<Pairs>(sm.tgt, col), row < h && col < z, cs);
                }
                float ctot;
                const float q = grp.scanf(r, ctot);
                const bool pos = (i < len) && (r > 0.0f);
                const int hit = grp.first(pos && q >= rem);
                if (hit >= 0) { chosen = kb + i0 + hit; break; }
                const int lp = grp.last(pos);
                if (lp >= 0) last_pos = kb + i0 + lp;
                rem -= ctot;
            }
        }
        if (chosen < 0) chosen = last_pos;
        if (chosen < 0) { status = KMC_ERR_NONFINITE; break; }
#if defined(KMC_DEBUG_CHECKS)
        if (B.select_mismatch && stored) {
            // the same selection with an FP64 scan and compare over the same
            // FP32 per-thread sums: count the hops where it picks another pair
            double dex, dtot;
            const double dinc = grp.scan_f64(static_cast<double>(lsum), dex, dtot);
            const double dtarget = __ull2double_rn(u_ev) * 0x1.0p-64 * dtot;
            int L64 = grp.first(dinc >= dtarget);
            if (L64 < 0) L64 = grp.last(run_e > run_b);
            const float rem64 = grp.bcast(static_cast<float>(dtarget - dex), L64);
            if (g == 0) {
                int kb64, ke64;
                run_of(L64, kb64, ke64);
                const int len = ke64 - kb64;
                int c64 = -1, lp = -1;
                for (int i = 0; i < len; ++i) {
                    const float ri = sm.rates[i * RS + L64];
                    if (c64 < 0 && ri >= (rem64 > 0.0f ? rem64 : 1.0e-38f)) c64 = i;
                    if (ri > (i > 0 ? sm.rates[(i - 1) * RS + L64] : 0.0f)) lp = i;
                }
                if (c64 < 0) c64 = lp;
                if (kb64 + c64 != chosen) B.select_mismatch[c] += 1ull;
            }
        }
#endif
        int row, col;
        KMC_DCHECK(chosen >= 0 && chosen < A && L >= 0 && L < G && chosen >= kbL && chosen < keL);
        decode_pair(chosen, h, A1, T1, T2, inv1, inv2, row, col);
        KMC_DCHECK(row >= 0 && row < h + P && col >= 0 && col < (row < h ? T1 : T2));
#ifdef KMC_DEBUG_CHECKS
        if (grp.first(dbg_bad != 0) >= 0) { status = KMC_ERR_INVALID; break; }
#endif
        const int from = Pairs::kSiteInRec ? Pairs::site(sm.src[row]) : sm.src_id[row];
        const int to = Pairs::kSiteInRec ? Pairs::site(tgt_load<Pairs>(sm.tgt, col)) : sm.tgt_id[col];
        KMC_DCHECK(from >= 0 && from < S && to >= 0 && to < S && from != to && (from < N || to < N));
#ifdef KMC_DEBUG_CHECKS
        if (grp.first(dbg_bad != 0) >= 0) { status = KMC_ERR_INVALID; break; }
#endif
        if (B.hop_log && g == 0) {
            const int64_t li = B.hop_log_off[c] + hop;
            B.hop_log[2 * li] = from;
            B.hop_log[2 * li + 1] = to;
            if (B.hop_rates) {
                B.hop_rates[2 * li] = totf;
                B.hop_rates[2 * li + 1] = pairs.rate(sm.src[row], tgt_load<Pairs>(sm.tgt, col), row < h && col < z, cs);
            }
        }
        KMC_SECTION(4);
        // ---- clock ----
        const float dt = e1 * rcp_approx(totf);
        const double t_before = t;
        t += static_cast<double>(dt);
        if (B.flux_time) {
            // Expected net hole flow into each electrode in this state,
            // J_e = sum_holes rate(i -> e) - sum_empty rate(e -> j), times
            // the time spent in it: the integral of J_e over the run is the
            // compensator of the electrode's hop count (their difference is
            // a zero-mean martingale), a low-variance companion estimate of
            // the current for accuracy checks.
            for (int e = 0; e < P; ++e) {
                const Rec er = sm.src[h + e];
                float part = 0.0f;
                for (int k = g; k < N; k += G)
                    part += (k < h) ? pairs.rate(sm.src[k], er, false, cs) : -pairs.rate(er, tgt_load<Pairs>(sm.tgt, k - h), false, cs);
                const float J = grp.sumf(part);
                if (g == 0) B.flux_time[eoff + e] += static_cast<double>(J) * static_cast<double>(dt);
            }
        }
        grp.sync();   // every thread is done reading the lists and rates
        KMC_SECTION(5);
        // ---- apply the hop and rebuild the lists in one pass ----
        const bool fa = from < N, tb = to < N;
        const int h_new = h + (tb ? 1 : 0) - (fa ? 1 : 0);
        const int z_new = N - h_new;
        {
            int wcur = 0, cum = 0;
            for (int j = g; j < N; j += G) {
                // O(N) update (makeJump, simulation.go:107-130), compensated
                float Ej = sm.E[j], Elo = kComp ? sm.Elo[j] : 0.0f;
                if (fa && j != from) eadd(Ej, Elo, -pairs.coulomb(j, from));
                if (tb && j != to) eadd(Ej, Elo, pairs.coulomb(j, to));
                sm.E[j] = Ej;
                if (kComp) sm.Elo[j] = Elo;
                const int w = j >> 5;
                while (wcur < w) { cum += __popc(sm.occw[wcur]); ++wcur; }
                const uint32_t word = sm.occw[w];
                // holes below j and the bit of j after the hop
                const int below = cum + __popc(word & ((1u << (j & 31)) - 1u))
                                  - ((fa && from < j) ? 1 : 0) + ((tb && to < j) ? 1 : 0);
                const bool occ_j = (j == to && tb) || (j != from && ((word >> (j & 31)) & 1u));
#ifdef KMC_DEBUG_CHECKS
                if (occ_j ? !(below >= 0 && below < h_new) : !(j - below >= 0 && j - below < z_new)) {
                    dbg_bad = 1;        // skip the store: the chain stops after this hop
                    continue;
                }
#endif
                const Rec r = pairs.rec(j, cs * (kComp ? Ej + Elo : Ej));
                if (occ_j) {
                    sm.src[below] = r;
                    if (!Pairs::kSiteInRec) sm.src_id[below] = j;
                } else {
                    tgt_store<Pairs>(sm.tgt, j - below, r);
                    if (!Pairs::kSiteInRec) sm.tgt_id[j - below] = j;
                }
            }
            if (h_new != h) {
                for (int e = g; e < P; e += G) {
                    const Rec r = (e == g) ? el_rec : pairs.rec(N + e, cs * Vel[e]);
                    sm.src[h_new + e] = r;
                    if (!Pairs::kSiteInRec) sm.src_id[h_new + e] = N + e;
                    tgt_store<Pairs>(sm.tgt, z_new + e, r);
                    if (!Pairs::kSiteInRec) sm.tgt_id[z_new + e] = N + e;
                }
            }
        }
        KMC_SECTION(6);
        grp.sync();   // lists complete; the bitmask is read no more this hop
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
        KMC_SECTION(7);
        h = h_new;
        ++hop;
#ifdef KMC_DEBUG_CHECKS
        if (grp.first(dbg_bad != 0) >= 0) { status = KMC_ERR_INVALID; break; }
#endif
    }
    grp.sync();

#ifdef KMC_SECTION_CLOCKS
    if (g == 0) {
        for (int k = 0; k < kSections; ++k) atomicAdd(&g_section_clocks[k], static_cast<unsigned long long>(sec_cycles[k]));
        atomicAdd(&g_section_clocks[kSections], static_cast<unsigned long long>(hop - hops_done0));
    }
#endif
    // ---- write back ----
    if (record) {
        const double td = t;
        for (int j = g; j < N; j += G)
            if ((sm.occw[j >> 5] >> (j & 31)) & 1u) {
                occ_time[j] += td - occ_since[j];
                occ_since[j] = td;
            }
    }
    for (int j = g; j < N; j += G) occ_g[j] = static_cast<uint8_t>((sm.occw[j >> 5] >> (j & 31)) & 1u);
    for (int e = g; e < P; e += G) B.electrode_occupation[eoff + e] += sm.eo[e];
    if (B.energy_drift) {
        // largest drift of the chain's threads, in kT (non-negative floats
        // order as their bit patterns)
        const float dm = __uint_as_float(grp.max_u32(__float_as_uint(drift_max * (cs / kLog2e))));
        if (g == 0) B.energy_drift[c] = fmaxf(B.energy_drift[c], dm);
    }
    if (g == 0) {
        B.time[c] = t;
        B.hops_done[c] = hop;
        B.status[c] = status;
        if (B.n_pairs) B.n_pairs[c] += npairs;
    }
}

// Stage the one pair table of a launch in shared memory (the whole block).
__device__ __forceinline__ const float2 *stage_table(const kmc_batch &B, uint32_t *smem, int table_words)
{
    if (table_words <= 0) return nullptr;
    // exactly the table's S*S (L, B) pairs; table_words only rounds the
    // shared-memory reservation up
    const int S = B.tab_N[0] + B.tab_P[0];
    if (S > B.max_sites) return nullptr;   // invalid launch: chains report it
    const float2 *src = reinterpret_cast<const float2 *>(B.tab_LB + B.tab_off[0]);
    float2 *dst = reinterpret_cast<float2 *>(smem);
    for (int i = threadIdx.x; i < S * S; i += blockDim.x) dst[i] = __ldg(&src[i]);
    __syncthreads();
    return reinterpret_cast<const float2 *>(smem);
}

// Stage the one pair table of a launch whose chains all have kT = kT_u as
// (L, fma(c, B, L)) pairs followed by the B values, c = log2(e)/kT_u.
__device__ __forceinline__ const float2 *stage_table_uniform(const kmc_batch &B, uint32_t *smem, int table_words)
{
    if (table_words <= 0) return nullptr;
    const int S = B.tab_N[0] + B.tab_P[0];
    if (S > B.max_sites) return nullptr;   // invalid launch: chains report it
    const float cu = kLog2e / B.uniform_kT;
    const float2 *src = reinterpret_cast<const float2 *>(B.tab_LB + B.tab_off[0]);
    float2 *dst = reinterpret_cast<float2 *>(smem);
    float *bdst = reinterpret_cast<float *>(dst + S * S);
    for (int i = threadIdx.x; i < S * S; i += blockDim.x) {
        const float2 lb = __ldg(&src[i]);
        dst[i] = make_float2(lb.x, fmaf(cu, lb.y, lb.x));
        bdst[i] = lb.y;
    }
    __syncthreads();
    return reinterpret_cast<const float2 *>(smem);
}

// Warp-sliced kernel: 32/G chains per warp, warps_per_block warps.  Two
// register budgets: MinBlocks = 3 blocks of 256 threads keeps registers at
// or below 85 so that 24 warps fit on an SM (launches with more blocks than
// the SMs hold at 2 each); MinBlocks = 2 allows 128 registers (16 warps per
// SM), which the pair walk uses without spills: 5.6 % faster on 4096 N=30
// chains, whose 256 blocks all fit.  table_words > 0: every chain of the
// launch uses table 0, staged in shared memory ahead of the per-chain areas.
template <int G, typename Pairs, int MinBlocks>
__global__ void __launch_bounds__(256, MinBlocks) warp_engine_kernel(const kmc_batch B, int rate_words,
                                                                     int table_words)
{
    constexpr int CPW = 32 / G;
    extern __shared__ __align__(16) uint32_t smem[];
    const float2 *stab = Pairs::kUniformTable ? stage_table_uniform(B, smem, table_words)
                                              : stage_table(B, smem, table_words);
    WarpGroup<G> grp;
    grp.init();
    const int warp = threadIdx.x >> 5;
    using Rec = typename Pairs::Rec;
    const int words = chain_list_words<Rec>(B.max_sites) + rate_words;
    ChainSmem<Rec> sm = carve<Rec>(smem + table_words + (warp * CPW + grp.sub) * words, B.max_sites,
                                   rate_words);
    if (B.work_counter) {
        // Persistent launch: each warp claims the next unclaimed item when
        // the chains of its last one are done, so a warp whose chains end
        // early takes more work instead of idling until its block ends.
        // Every lane of the warp takes part in each claim (an item with an
        // empty slot leaves that group idle until the next claim), and the
        // loop ends for the whole warp at once, when the list is used up.
        const int lane = threadIdx.x & 31;
        for (;;) {
            int item = 0;
            if (lane == 0) item = atomicAdd(B.work_counter, 1);
            item = __shfl_sync(0xffffffffu, item, 0);
            if (item >= B.n_work) break;
            const int c = B.work[item * CPW + grp.sub];
            if (c >= 0 && c < B.n_chains) run_chain<WarpGroup<G>, Pairs>(B, grp, sm, c, stab);
            __syncwarp();
        }
        return;
    }
    const int item = blockIdx.x * B.warps_per_block + warp;
    if (item >= B.n_work) return;
    const int c = B.work[item * CPW + grp.sub];
    if (c < 0 || c >= B.n_chains) return;   // the whole group leaves together
    run_chain<WarpGroup<G>, Pairs>(B, grp, sm, c, stab);
}

// Block kernel: one chain per block of T threads.
template <int T, typename Pairs>
__global__ void __launch_bounds__(T) block_engine_kernel(const kmc_batch B, int rate_words,
                                                         int table_words)
{
    extern __shared__ __align__(16) uint32_t smem[];
    __shared__ double scratch[T / 32 + 2];
    __shared__ int iscratch[2];
    const float2 *stab = stage_table(B, smem, table_words);
    BlockGroup<T> grp;
    grp.init();
    grp.sd = scratch;
    grp.si = iscratch;
    using Rec = typename Pairs::Rec;
    ChainSmem<Rec> sm = carve<Rec>(smem + table_words, B.max_sites, rate_words);
    if (B.work_counter) {
        // Persistent launch: the block claims the next chain when its last
        // one is done.
        for (;;) {
            if (threadIdx.x == 0) iscratch[0] = atomicAdd(B.work_counter, 1);
            __syncthreads();
            const int item = iscratch[0];
            __syncthreads();
            if (item >= B.n_work) break;
            const int c = B.work[item];
            if (c >= 0 && c < B.n_chains) run_chain<BlockGroup<T>, Pairs>(B, grp, sm, c, stab);
            __syncthreads();
        }
        return;
    }
    const int c = B.work[blockIdx.x];
    if (c < 0 || c >= B.n_chains) return;   // uniform over the block
    run_chain<BlockGroup<T>, Pairs>(B, grp, sm, c, stab);
}

template <typename K>
int set_smem(K kernel, size_t smem, int &configured)
{
    // Raise the dynamic shared-memory limit only when a launch needs more
    // than any before it, so launches under stream capture make no
    // attribute calls once a first launch has run.
    if (static_cast<int>(smem) > configured) {
        cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(smem));
        if (e != cudaSuccess) return fail_cuda(e, "cudaFuncSetAttribute(engine)");
        configured = static_cast<int>(smem);
    }
    return KMC_OK;
}

// SMs of the current device (queried once).
int sm_count()
{
    static int n = 0;
    if (n == 0) {
        int dev = 0, v = 0;
        if (cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && v > 0)
            n = v;
        else
            return 1;
    }
    return n;
}

constexpr size_t kSmemBudget = 200 * 1024;   // per block, leaving room for static scratch

// Words of the staged pair table, or 0 when the launch has more than one
// table (or is not in table mode) or it would not fit next to `rest` bytes.
template <typename Pairs>
int table_stage_words(const kmc_batch &b, size_t rest)
{
    if (b.pair_mode != KMC_PAIRS_TABLE || b.n_tables != 1) return 0;
    const size_t w = ((2 * static_cast<size_t>(b.max_sites) * b.max_sites) + 3) & ~static_cast<size_t>(3);
    return (w * 4 + rest <= kSmemBudget && w * 4 <= 64 * 1024) ? static_cast<int>(w) : 0;
}

template <int G, typename Pairs>
int launch_warp_kernel(const kmc_batch &b, cudaStream_t st, int grid, size_t smem, int rw, int tw)
{
    // The register-rich variant when every block of the launch is resident
    // at once with 16 warps per SM, else the one that fits 24.
    const int wpb = b.warps_per_block;
    const int rich_blocks = (16 / wpb) * sm_count();
    if (b.work_counter) {
        // persistent: as many blocks as stay resident at once (85-register
        // variant), no more than the work needs
        static int configured_p = 0;
        const int rc = set_smem(warp_engine_kernel<G, Pairs, 3>, smem, configured_p);
        if (rc != KMC_OK) return rc;
        int per_sm = 0;
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, warp_engine_kernel<G, Pairs, 3>,
                                                                      wpb * 32, smem);
        if (e != cudaSuccess) return fail_cuda(e, "engine occupancy");
        int pgrid = min(grid, max(1, per_sm) * sm_count());
        if (b.max_grid > 0) pgrid = min(pgrid, b.max_grid);
        warp_engine_kernel<G, Pairs, 3><<<pgrid, wpb * 32, smem, st>>>(b, rw, tw);
        e = cudaGetLastError();
        return e == cudaSuccess ? KMC_OK : fail_cuda(e, "engine launch");
    }
    if (grid <= rich_blocks) {
        static int configured_rich = 0;
        const int rc = set_smem(warp_engine_kernel<G, Pairs, 2>, smem, configured_rich);
        if (rc != KMC_OK) return rc;
        warp_engine_kernel<G, Pairs, 2><<<grid, wpb * 32, smem, st>>>(b, rw, tw);
    } else {
        static int configured = 0;
        const int rc = set_smem(warp_engine_kernel<G, Pairs, 3>, smem, configured);
        if (rc != KMC_OK) return rc;
        warp_engine_kernel<G, Pairs, 3><<<grid, wpb * 32, smem, st>>>(b, rw, tw);
    }
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? KMC_OK : fail_cuda(e, "engine launch");
}

template <int G, typename Pairs>
int preload_warp_kernels()
{
    int rc;
    if ((rc = touch_kernel(warp_engine_kernel<G, Pairs, 2>)) != KMC_OK) return rc;
    return touch_kernel(warp_engine_kernel<G, Pairs, 3>);
}
template <int G, typename Pairs>
int launch_warp(const kmc_batch &b, cudaStream_t st)
{
    constexpr int CPW = 32 / G;
    const int wpb = b.warps_per_block;
    const int lw = chain_list_words<typename Pairs::Rec>(b.max_sites);
    int rw = rate_buffer_words(b.max_sites, G);
    // Pad each chain's area to G words modulo 32: the 32/G chains of a warp
    // then store their running sums (row i of the transposed layout) to
    // disjoint banks.
    if (G < 32) rw += ((G - (lw + rw)) % 32 + 32) % 32;
    if (static_cast<size_t>(wpb) * CPW * (lw + rw) * 4 > kSmemBudget) rw = 0;   // recompute instead
    const size_t chains = static_cast<size_t>(wpb) * CPW * (lw + rw) * 4;
    const int tw = table_stage_words<Pairs>(b, chains);
    const size_t smem = chains + static_cast<size_t>(tw) * 4;
    if (smem > kSmemBudget)
        return fail(KMC_ERR_INVALID, "engine: %zu bytes of shared memory per block (max_sites %d, G %d, %d warps) exceeds the budget",
                    smem, b.max_sites, G, wpb);
    const int grid = (b.n_work + wpb - 1) / wpb;
    if (grid <= 0) return KMC_OK;
    if (tw > 0 && b.uniform_kT > 0.0f) {
        // every chain has kT = uniform_kT: stage (L, L + c B) and B (3 S^2 words)
        const int tw3 = ((3 * b.max_sites * b.max_sites) + 3) & ~3;
        const size_t smem3 = chains + static_cast<size_t>(tw3) * 4;
        if (smem3 <= kSmemBudget && static_cast<size_t>(tw3) * 4 <= 96 * 1024)
            return launch_warp_kernel<G, TablePairs<true, true>>(b, st, grid, smem3, rw, tw3);
    }
    if (tw > 0) return launch_warp_kernel<G, TablePairs<true>>(b, st, grid, smem, rw, tw);
    return launch_warp_kernel<G, Pairs>(b, st, grid, smem, rw, tw);
}

template <int T, typename Pairs>
int launch_block_kernel(const kmc_batch &b, cudaStream_t st, size_t smem, int rw, int tw)
{
    static int configured = 0;
    const int rc = set_smem(block_engine_kernel<T, Pairs>, smem, configured);
    if (rc != KMC_OK) return rc;
    if (b.n_work <= 0) return KMC_OK;
    int grid = b.n_work;
    if (b.work_counter) {   // persistent: the resident blocks claim the chains
        int per_sm = 0;
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, block_engine_kernel<T, Pairs>, T, smem);
        if (e != cudaSuccess) return fail_cuda(e, "engine occupancy");
        grid = min(grid, max(1, per_sm) * sm_count());
        if (b.max_grid > 0) grid = min(grid, b.max_grid);
    }
    block_engine_kernel<T, Pairs><<<grid, T, smem, st>>>(b, rw, tw);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? KMC_OK : fail_cuda(e, "engine launch");
}

template <int T, typename Pairs>
int preload_block_kernel()
{
    return touch_kernel(block_engine_kernel<T, Pairs>);
}
template <int T, typename Pairs>
int launch_block(const kmc_batch &b, cudaStream_t st)
{
    const int lw = chain_list_words<typename Pairs::Rec>(b.max_sites);
    int rw = rate_buffer_words(b.max_sites, T);
    if (static_cast<size_t>(lw + rw) * 4 > kSmemBudget) rw = 0;
    if (rw > 0) {
        // Without the running-sum buffer the event search re-evaluates the
        // chosen thread's run, for a block group a chunk or two of rates.
        // Drop the buffer when it is what limits the blocks an SM holds and
        // the launch has more chains than the SMs then hold at once (a
        // 512-chain request of N=240 networks at 512 threads: one wave of
        // blocks instead of two).
        const int per_sm_threads = 2048 / T;
        const int per_sm_with = static_cast<int>((227 * 1024) / (static_cast<size_t>(lw + rw) * 4));
        const int per_sm_without = static_cast<int>((227 * 1024) / (static_cast<size_t>(lw) * 4));
        if (per_sm_with < per_sm_threads && per_sm_without > per_sm_with &&
            b.n_work > per_sm_with * sm_count())
            rw = 0;
    }
    const size_t chain = static_cast<size_t>(lw + rw) * 4;
    const int tw = table_stage_words<Pairs>(b, chain);
    const size_t smem = chain + static_cast<size_t>(tw) * 4;
    if (smem > kSmemBudget)
        return fail(KMC_ERR_INVALID, "engine: %zu bytes of shared memory per chain (max_sites %d) exceeds the block budget",
                    smem, b.max_sites);
    if (tw > 0) return launch_block_kernel<T, TablePairs<true>>(b, st, smem, rw, tw);
    return launch_block_kernel<T, Pairs>(b, st, smem, rw, tw);
}

}  // namespace
}  // namespace kmc
