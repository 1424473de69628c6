// kmc_laplace.cu -- Laplace basis fields on the device.
//
// The potential of a network is a superposition of unit-voltage solutions
// of the Laplace problem on its mesh (init_V / update_V,
// kmc_dopant_networks.py:706-822, solve P1 elements with Dirichlet data on
// the whole boundary).  On the uniform right-triangle mesh the P1 system is
// the anisotropic 5-point stencil
//     (2cx + 2cy) u_ij - cx (u_i,j-1 + u_i,j+1) - cy (u_i-1,j + u_i+1,j) = 0,
// cx = hy/hx, cy = hx/hy, whose matrix cx (I ⊗ T_x) + cy (T_y ⊗ I), with
// T = tridiag(-1, 2, -1), is diagonalised by discrete sine transforms:
//     T_n = Q_n diag(lambda) Q_n,  Q_n[a][b] = sqrt(2/n) sin(pi (a+1)(b+1)/n),
//     lambda_b = 2 - 2 cos(pi (b+1)/n)   (n = cells, size n-1).
// So U = Q_y ((Q_y F Q_x) ./ (cx lambda_x + cy lambda_y)) Q_x, F the
// right-hand side carrying the boundary data: four small FP64 matrix
// products per field, exact up to rounding (no iteration, no tolerance).
// All fields of one mesh are solved in one batch; P1 sampling at the
// acceptors follows.  This replaces the per-geometry CPU solve when
// geometries churn (serving).
#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>

#include "kmc_internal.h"

namespace kmc {
namespace {

constexpr int kTile = 16;

// Q[a][b] = sqrt(2/n) sin(pi (a+1)(b+1)/n), (n-1) x (n-1); lam[b].
__global__ void dst_basis_kernel(int n, double *Q, double *lam)
{
    const int m = n - 1;
    const double pi = 3.14159265358979323846;
    const double s = sqrt(2.0 / n);
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < m * m; k += gridDim.x * blockDim.x) {
        const int a = k / m, b = k - (k / m) * m;
        // (a+1)(b+1) mod 2n keeps the sine argument small and exact
        const long long p = (static_cast<long long>(a + 1) * (b + 1)) % (2LL * n);
        Q[k] = s * sin(pi * static_cast<double>(p) / n);
        if (a == 0) lam[b] = 2.0 - 2.0 * cos(pi * (b + 1) / n);
    }
}

// Right-hand side of the interior system from the boundary values of each
// field's nodal grid ((ny+1) x (nx+1), row = y index).
__global__ void rhs_kernel(int nx, int ny, double cx, double cy, int nf, const double *grid, double *F)
{
    const int mi = ny - 1, mj = nx - 1;
    const long long per = static_cast<long long>(mi) * mj;
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < per * nf;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int f = static_cast<int>(k / per);
        const long long r = k - f * per;
        const int i = static_cast<int>(r / mj) + 1, j = static_cast<int>(r % mj) + 1;   // node indices
        const double *g = grid + static_cast<long long>(f) * (ny + 1) * (nx + 1);
        double b = 0.0;
        if (j == 1) b += cx * g[i * (nx + 1) + 0];
        if (j == nx - 1) b += cx * g[i * (nx + 1) + nx];
        if (i == 1) b += cy * g[0 * (nx + 1) + j];
        if (i == ny - 1) b += cy * g[ny * (nx + 1) + j];
        F[k] = b;
    }
}

// C_f = op(A) * B_f or B_f * op(A) for every field f (blockIdx.z), FP64,
// shared-memory tiles.  left: C = A (m x m) * X (m x n); else C = X (m x n) * A (n x n).
__global__ void gemm_kernel(int m, int n, const double *A, const double *X, double *C, int left)
{
    __shared__ double ta[kTile][kTile + 1];
    __shared__ double tb[kTile][kTile + 1];
    const long long off = static_cast<long long>(blockIdx.z) * m * n;
    const double *Xf = X + off;
    double *Cf = C + off;
    const int row = blockIdx.y * kTile + threadIdx.y;
    const int col = blockIdx.x * kTile + threadIdx.x;
    const int K = left ? m : n;
    double acc = 0.0;
    for (int k0 = 0; k0 < K; k0 += kTile) {
        const int ka = k0 + threadIdx.x, kb = k0 + threadIdx.y;
        if (left) {
            ta[threadIdx.y][threadIdx.x] = (row < m && ka < K) ? A[row * m + ka] : 0.0;
            tb[threadIdx.y][threadIdx.x] = (kb < K && col < n) ? Xf[kb * n + col] : 0.0;
        } else {
            ta[threadIdx.y][threadIdx.x] = (row < m && ka < K) ? Xf[row * n + ka] : 0.0;
            tb[threadIdx.y][threadIdx.x] = (kb < K && col < n) ? A[kb * n + col] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kTile; ++k) acc = fma(ta[threadIdx.y][k], tb[k][threadIdx.x], acc);
        __syncthreads();
    }
    if (row < m && col < n) Cf[row * n + col] = acc;
}

__global__ void scale_kernel(int mi, int mj, double cx, double cy, const double *lamx, const double *lamy,
                             int nf, double *W)
{
    const long long per = static_cast<long long>(mi) * mj;
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < per * nf;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const long long r = k % per;
        const int l = static_cast<int>(r / mj), kk = static_cast<int>(r % mj);
        W[k] /= (cx * lamx[kk] + cy * lamy[l]);
    }
}

__global__ void scatter_kernel(int nx, int ny, int nf, const double *U, double *grid)
{
    const int mi = ny - 1, mj = nx - 1;
    const long long per = static_cast<long long>(mi) * mj;
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < per * nf;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int f = static_cast<int>(k / per);
        const long long r = k - f * per;
        const int i = static_cast<int>(r / mj) + 1, j = static_cast<int>(r % mj) + 1;
        grid[static_cast<long long>(f) * (ny + 1) * (nx + 1) + i * (nx + 1) + j] = U[k];
    }
}

// P1 interpolation on the "right" diagonal triangulation (ix,iy)-(ix+1,iy+1).
__global__ void p1_sample_kernel(int nx, int ny, double hx, double hy, int nf, const double *grid,
                                 int np, const double *xy, double *out)
{
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
         k < static_cast<long long>(np) * nf; k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int f = static_cast<int>(k / np), p = static_cast<int>(k - static_cast<long long>(f) * np);
        const double sx = xy[2 * p] / hx, sy = xy[2 * p + 1] / hy;
        int ix = static_cast<int>(floor(sx)), iy = static_cast<int>(floor(sy));
        ix = ix < 0 ? 0 : (ix > nx - 1 ? nx - 1 : ix);
        iy = iy < 0 ? 0 : (iy > ny - 1 ? ny - 1 : iy);
        const double xi = sx - ix, eta = sy - iy;
        const double *g = grid + static_cast<long long>(f) * (ny + 1) * (nx + 1);
        const double f00 = g[iy * (nx + 1) + ix], f10 = g[iy * (nx + 1) + ix + 1];
        const double f01 = g[(iy + 1) * (nx + 1) + ix], f11 = g[(iy + 1) * (nx + 1) + ix + 1];
        out[k] = (xi >= eta) ? f00 + xi * (f10 - f00) + eta * (f11 - f10)
                             : f00 + eta * (f01 - f00) + xi * (f11 - f01);
    }
}

int grid_for(long long n)
{
    const long long b = (n + 255) / 256;
    return static_cast<int>(b < 1 ? 1 : (b > 4096 ? 4096 : b));
}

}  // namespace
}  // namespace kmc

using namespace kmc;

extern "C" size_t kmc_laplace_workspace_size(int32_t nx, int32_t ny, int32_t n_fields)
{
    if (nx < 2 || ny < 2 || n_fields < 1) return 0;
    const size_t mi = ny - 1, mj = nx - 1;
    return sizeof(double) * (mi * mi + mj * mj + mi + mj + 2 * mi * mj * static_cast<size_t>(n_fields));
}

extern "C" int kmc_laplace_basis(int32_t nx, int32_t ny, double hx, double hy, int32_t n_fields,
                                 double *grid, void *workspace, size_t workspace_bytes, void *stream)
{
    if (nx < 2 || ny < 2 || n_fields < 1 || !(hx > 0) || !(hy > 0))
        return fail(KMC_ERR_INVALID, "laplace_basis: bad mesh (nx %d, ny %d, fields %d)", nx, ny, n_fields);
    if (!grid || !workspace) return fail(KMC_ERR_INVALID, "laplace_basis: NULL pointer");
    if (workspace_bytes < kmc_laplace_workspace_size(nx, ny, n_fields))
        return fail(KMC_ERR_INVALID, "laplace_basis: workspace too small");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int mi = ny - 1, mj = nx - 1;
    double *Qy = static_cast<double *>(workspace);
    double *Qx = Qy + static_cast<size_t>(mi) * mi;
    double *ly = Qx + static_cast<size_t>(mj) * mj;
    double *lx = ly + mi;
    double *W1 = lx + mj;
    double *W2 = W1 + static_cast<size_t>(mi) * mj * n_fields;
    const double cx = hy / hx, cy = hx / hy;
    dst_basis_kernel<<<grid_for(static_cast<long long>(mi) * mi), 256, 0, st>>>(ny, Qy, ly);
    dst_basis_kernel<<<grid_for(static_cast<long long>(mj) * mj), 256, 0, st>>>(nx, Qx, lx);
    const long long tot = static_cast<long long>(mi) * mj * n_fields;
    rhs_kernel<<<grid_for(tot), 256, 0, st>>>(nx, ny, cx, cy, n_fields, grid, W1);
    const dim3 blk(kTile, kTile), grd((mj + kTile - 1) / kTile, (mi + kTile - 1) / kTile, n_fields);
    gemm_kernel<<<grd, blk, 0, st>>>(mi, mj, Qy, W1, W2, 1);      // Qy F
    gemm_kernel<<<grd, blk, 0, st>>>(mi, mj, Qx, W2, W1, 0);      // (Qy F) Qx
    scale_kernel<<<grid_for(tot), 256, 0, st>>>(mi, mj, cx, cy, lx, ly, n_fields, W1);
    gemm_kernel<<<grd, blk, 0, st>>>(mi, mj, Qy, W1, W2, 1);
    gemm_kernel<<<grd, blk, 0, st>>>(mi, mj, Qx, W2, W1, 0);
    scatter_kernel<<<grid_for(tot), 256, 0, st>>>(nx, ny, n_fields, W1, grid);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? KMC_OK : fail_cuda(e, "laplace_basis launch");
}

extern "C" int kmc_p1_sample(int32_t nx, int32_t ny, double hx, double hy, int32_t n_fields,
                             const double *grid, int32_t n_points, const double *xy, double *out,
                             void *stream)
{
    if (nx < 1 || ny < 1 || n_fields < 1 || n_points < 0 || !(hx > 0) || !(hy > 0))
        return fail(KMC_ERR_INVALID, "p1_sample: bad sizes");
    if (n_points == 0) return KMC_OK;
    if (!grid || !xy || !out) return fail(KMC_ERR_INVALID, "p1_sample: NULL pointer");
    const long long tot = static_cast<long long>(n_points) * n_fields;
    p1_sample_kernel<<<grid_for(tot), 256, 0, static_cast<cudaStream_t>(stream)>>>(nx, ny, hx, hy, n_fields,
                                                                                 grid, n_points, xy, out);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? KMC_OK : fail_cuda(e, "p1_sample launch");
}

namespace kmc {

int preload_laplace()
{
    int rc;
    if ((rc = touch_kernel(dst_basis_kernel)) != KMC_OK) return rc;
    if ((rc = touch_kernel(rhs_kernel)) != KMC_OK) return rc;
    if ((rc = touch_kernel(gemm_kernel)) != KMC_OK) return rc;
    if ((rc = touch_kernel(scale_kernel)) != KMC_OK) return rc;
    if ((rc = touch_kernel(scatter_kernel)) != KMC_OK) return rc;
    return touch_kernel(p1_sample_kernel);
}

}  // namespace kmc
