// kmc_internal.h -- host-side helpers shared by the translation units.
#pragma once
#include <cuda_runtime.h>

#include "../../include/kmc_dn_gb300.h"

namespace kmc {

// Largest site count the batched engine accepts: keeps the number of pairs
// A(h) < 2^22 (exact float-reciprocal pair decoding) and the per-chain
// shared-memory lists within one block.
constexpr int kMaxSitesF32 = 2048;
// Largest site count of the plain FP64 kernel.
constexpr int kMaxSitesF64 = 2048;

// Record an error for kmc_last_error and return its code.
int fail(int code, const char *fmt, ...);
int fail_cuda(cudaError_t e, const char *what);
int ok();

int run_batch(const kmc_batch &b, cudaStream_t st);
// engine launches by group kind and pair mode (kmc_f32_*.cu)
int launch_warp_table(const kmc_batch &b, cudaStream_t st);
int launch_warp_positions(const kmc_batch &b, cudaStream_t st);
int launch_block_table(const kmc_batch &b, cudaStream_t st);
int launch_block_positions(const kmc_batch &b, cudaStream_t st);
int section_clocks_warp_table(uint64_t *out, int reset);
int section_clocks_warp_positions(uint64_t *out, int reset);
int section_clocks_block(uint64_t *out, int reset);
// Load every kernel of a translation unit (kmc_preload_kernels).
int preload_warp_table();
int preload_warp_positions();
int preload_block();
int preload_f64();
int preload_setup();
int preload_meanfield();
int preload_laplace();
// Force the module loading of one kernel now (a kernel loaded lazily at its
// first launch waits for the kernels already running on the device).
template <typename K>
inline int touch_kernel(K *kernel)
{
    cudaFuncAttributes a;
    const cudaError_t e = cudaFuncGetAttributes(&a, reinterpret_cast<const void *>(kernel));
    return e == cudaSuccess ? KMC_OK : fail_cuda(e, "kernel preload");
}
// Per-phase cycle counters of a -DKMC_SECTION_CLOCKS build (9 values).
int section_clocks(uint64_t *out, int reset);
int build_table(int N, int P, double nu, double I0, double R, const double *d, const double *tc,
                float *tab, cudaStream_t st);
int site_energies(int n_chains, int N, int P, const double *basis, const double *V, double mu,
                  const double *comp, float *Ec, float *Vel, cudaStream_t st);
int simulate_f64(int N, int P, double nu, double kT, double I0, double R, uint8_t *occ,
                 const double *d, const double *Ec, const double *se, const double *tc,
                 int64_t *eo, int64_t hops, int record, double *traffic, double *oit,
                 const double *uniforms, uint64_t seed, int32_t *hop_log, double *time_out,
                 int32_t *status_out, void *ws, size_t ws_bytes, cudaStream_t st,
                 double *flux_time = nullptr);
size_t f64_workspace_size(int S);
size_t f64_batch_workspace_size(int n_chains, int max_sites);
int simulate_f64_batch(const kmc_f64_batch &b, cudaStream_t st);

// Host-buffer batch run (FP64 host inputs, copies in/out, synchronous).
struct HostRun {
    int32_t n_geoms;
    const int32_t *geom_N, *geom_P;
    const double *geom_nu, *geom_I0, *geom_R;
    const int64_t *geom_pair_off;
    const double *distances, *transitions_constant;
    int32_t n_chains;
    const int32_t *chain_geom;
    const double *chain_kT, *E_constant, *site_energies;
    uint8_t *occupation;
    const int64_t *hops;
    const uint64_t *streams;        // NULL: chain index
    uint64_t seed;
    int32_t lanes_per_chain;
    int32_t record;                 // KMC_RECORD_*
    double *time_out;
    int64_t *electrode_occupation;  // overwritten
    int32_t *status;
    double *traffic_out;            // record: S*S per chain, accumulated
    double *occ_time_out;           // record: N per chain, accumulated
};
int host_run(const HostRun &h);

}  // namespace kmc
