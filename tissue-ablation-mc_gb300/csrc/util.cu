// util.cu -- set-up fills, layout conversions between the reference's halo
// layout and the interior state, and small reductions.
#include "tam_device.cuh"
#include "tam_util.h"

#include <atomic>

#include "tam_kernels.h"

namespace tam {

namespace {
std::atomic<int64_t> g_launches{0};
}  // namespace

void count_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
int64_t launch_count() { return g_launches.load(std::memory_order_relaxed); }

namespace {

int blocks_for(int64_t n, int tpb)
{
    int64_t b = (n + tpb - 1) / tpb;
    if (b > 152 * 16) b = 152 * 16;
    return (int)(b > 0 ? b : 1);
}

#define GRID_STRIDE(q, n) \
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < (n); q += (int64_t)gridDim.x * blockDim.x)

__global__ void fill_f64_kernel(double *p, double v, int64_t n)
{
    GRID_STRIDE(q, n) p[q] = v;
}
__global__ void fill_f32_kernel(float *p, float v, int64_t n)
{
    GRID_STRIDE(q, n) p[q] = v;
}
__global__ void fill_u8_kernel(uint8_t *p, uint8_t v, int64_t n)
{
    GRID_STRIDE(q, n) p[q] = v;
}

// interior -> vin; plane k == nz+1 -> vtop (when has_top); other halo -> vhalo
__global__ void fill_halo_kernel(double *p, int nx, int ny, int nz, double vin, double vhalo, double vtop,
                                 int has_top)
{
    const int64_t hx = nx + 2, hy = ny + 2, n = hx * hy * (nz + 2);
    GRID_STRIDE(q, n)
    {
        const int i = (int)(q % hx);
        const int j = (int)((q / hx) % hy);
        const int k = (int)(q / (hx * hy));
        double v;
        if (i >= 1 && i <= nx && j >= 1 && j <= ny && k >= 1 && k <= nz) v = vin;
        else if (has_top && k == nz + 1) v = vtop;
        else v = vhalo;
        p[q] = v;
    }
}

// src/mcpolar.f90:123-129: 5 C everywhere, 25 C on the z faces (assigned last)
__global__ void ref_init_temp_kernel(double *p, int nx, int ny, int nz)
{
    const int64_t hx = nx + 2, hy = ny + 2, n = hx * hy * (nz + 2);
    GRID_STRIDE(q, n)
    {
        const int k = (int)(q / (hx * hy));
        p[q] = (k == 0 || k == nz + 1) ? 25.0 + 273.0 : 5.0 + 273.0;
    }
}

template <typename Real>
__global__ void props_from_mat_kernel(const uint8_t *mat, int nmat, MatThermal lut, Real *k, Real *r, Real *c,
                                      int64_t n)
{
    GRID_STRIDE(q, n)
    {
        int m = mat[q];
        if (m >= nmat) m = 0;
        k[q] = (Real)lut.k[m];
        r[q] = (Real)lut.rho[m];
        c[q] = (Real)lut.c[m];
    }
}

template <typename Real> __global__ void to_f64_kernel(const Real *s, double *d, int64_t n)
{
    GRID_STRIDE(q, n) d[q] = (double)s[q];
}
template <typename Real> __global__ void from_f64_kernel(const double *s, Real *d, int64_t n)
{
    GRID_STRIDE(q, n) d[q] = (Real)s[q];
}

// interior (Real) -> halo double, ghosts copy the nearest interior value
template <typename Real>
__global__ void interior_to_halo_kernel(const Real *s, double *h, int nx, int ny, int nz)
{
    const int64_t hx = nx + 2, hy = ny + 2, n = hx * hy * (nz + 2);
    GRID_STRIDE(q, n)
    {
        const int i = (int)(q % hx), j = (int)((q / hx) % hy), k = (int)(q / (hx * hy));
        const int ci = min(max(i, 1), nx) - 1, cj = min(max(j, 1), ny) - 1, ck = min(max(k, 1), nz) - 1;
        h[q] = (double)s[(int64_t)ci + (int64_t)nx * ((int64_t)cj + (int64_t)ny * ck)];
    }
}

template <typename Real>
__global__ void halo_to_interior_kernel(const double *h, Real *s, int nx, int ny, int nz)
{
    const int64_t n = (int64_t)nx * ny * nz;
    GRID_STRIDE(q, n)
    {
        const int i = (int)(q % nx), j = (int)((q / nx) % ny), k = (int)(q / ((int64_t)nx * ny));
        s[q] = (Real)h[(int64_t)(i + 1) + (int64_t)(nx + 2) * ((int64_t)(j + 1) + (int64_t)(ny + 2) * (k + 1))];
    }
}

__global__ void rhokap_from_mat_kernel(const uint8_t *mat, int nmat, MatThermal lut, double *h, int nx, int ny,
                                       int nz)
{
    const int64_t hx = nx + 2, hy = ny + 2, n = hx * hy * (nz + 2);
    GRID_STRIDE(q, n)
    {
        const int i = (int)(q % hx), j = (int)((q / hx) % hy), k = (int)(q / (hx * hy));
        double v = 0.0;
        if (i >= 1 && i <= nx && j >= 1 && j <= ny && k >= 1 && k <= nz) {
            int m = mat[(int64_t)(i - 1) + (int64_t)nx * ((int64_t)(j - 1) + (int64_t)ny * (k - 1))];
            if (m >= nmat) m = 0;
            v = lut.mut[m];
        }
        h[q] = v;
    }
}

// min / max of rhokap-like halo array over the interior (validation helper)
__global__ void count_negative_kernel(const double *p, int64_t n, unsigned long long *out)
{
    unsigned long long c = 0;
    GRID_STRIDE(q, n) c += (p[q] < 0.0 || p[q] != p[q]) ? 1ull : 0ull;
    if (c) atomicAdd(out, c);
}

}  // namespace

cudaError_t launch_fill_f64(double *p, double v, int64_t n, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    count_launch();
    fill_f64_kernel<<<blocks_for(n, 256), 256, 0, s>>>(p, v, n);
    return cudaGetLastError();
}
cudaError_t launch_fill_real(void *p, bool fp64, double v, int64_t n, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    count_launch();
    if (fp64) fill_f64_kernel<<<blocks_for(n, 256), 256, 0, s>>>((double *)p, v, n);
    else fill_f32_kernel<<<blocks_for(n, 256), 256, 0, s>>>((float *)p, (float)v, n);
    return cudaGetLastError();
}
cudaError_t launch_fill_u8(uint8_t *p, uint8_t v, int64_t n, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    count_launch();
    fill_u8_kernel<<<blocks_for(n, 256), 256, 0, s>>>(p, v, n);
    return cudaGetLastError();
}
cudaError_t launch_fill_halo(double *p, int nx, int ny, int nz, double vin, double vhalo, double vtop, bool has_top,
                             cudaStream_t s)
{
    const int64_t n = (int64_t)(nx + 2) * (ny + 2) * (nz + 2);
    count_launch();
    fill_halo_kernel<<<blocks_for(n, 256), 256, 0, s>>>(p, nx, ny, nz, vin, vhalo, vtop, has_top ? 1 : 0);
    return cudaGetLastError();
}
cudaError_t launch_ref_init_temp(double *p, int nx, int ny, int nz, cudaStream_t s)
{
    const int64_t n = (int64_t)(nx + 2) * (ny + 2) * (nz + 2);
    count_launch();
    ref_init_temp_kernel<<<blocks_for(n, 256), 256, 0, s>>>(p, nx, ny, nz);
    return cudaGetLastError();
}
cudaError_t launch_props_from_mat(const uint8_t *mat, int nmat, const MatThermal &lut, void *k, void *r, void *c,
                                  bool fp64, int64_t n, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    count_launch();
    if (fp64)
        props_from_mat_kernel<double>
            <<<blocks_for(n, 256), 256, 0, s>>>(mat, nmat, lut, (double *)k, (double *)r, (double *)c, n);
    else
        props_from_mat_kernel<float>
            <<<blocks_for(n, 256), 256, 0, s>>>(mat, nmat, lut, (float *)k, (float *)r, (float *)c, n);
    return cudaGetLastError();
}
cudaError_t launch_to_f64(const void *src, bool fp64, double *dst, int64_t n, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    if (fp64) return cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToDevice, s);
    count_launch();
    to_f64_kernel<float><<<blocks_for(n, 256), 256, 0, s>>>((const float *)src, dst, n);
    return cudaGetLastError();
}
cudaError_t launch_from_f64(const double *src, void *dst, bool fp64, int64_t n, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    if (fp64) return cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToDevice, s);
    count_launch();
    from_f64_kernel<float><<<blocks_for(n, 256), 256, 0, s>>>(src, (float *)dst, n);
    return cudaGetLastError();
}
cudaError_t launch_interior_to_halo(const void *src, bool fp64, double *halo, int nx, int ny, int nz, cudaStream_t s)
{
    const int64_t n = (int64_t)(nx + 2) * (ny + 2) * (nz + 2);
    count_launch();
    if (fp64) interior_to_halo_kernel<double><<<blocks_for(n, 256), 256, 0, s>>>((const double *)src, halo, nx, ny, nz);
    else interior_to_halo_kernel<float><<<blocks_for(n, 256), 256, 0, s>>>((const float *)src, halo, nx, ny, nz);
    return cudaGetLastError();
}
cudaError_t launch_halo_to_interior(const double *halo, void *dst, bool fp64, int nx, int ny, int nz, cudaStream_t s)
{
    const int64_t n = (int64_t)nx * ny * nz;
    count_launch();
    if (fp64) halo_to_interior_kernel<double><<<blocks_for(n, 256), 256, 0, s>>>(halo, (double *)dst, nx, ny, nz);
    else halo_to_interior_kernel<float><<<blocks_for(n, 256), 256, 0, s>>>(halo, (float *)dst, nx, ny, nz);
    return cudaGetLastError();
}
cudaError_t launch_rhokap_from_mat(const uint8_t *mat, int nmat, const MatThermal &lut, double *halo, int nx, int ny,
                                   int nz, cudaStream_t s)
{
    const int64_t n = (int64_t)(nx + 2) * (ny + 2) * (nz + 2);
    count_launch();
    rhokap_from_mat_kernel<<<blocks_for(n, 256), 256, 0, s>>>(mat, nmat, lut, halo, nx, ny, nz);
    return cudaGetLastError();
}
cudaError_t launch_count_negative(const double *p, int64_t n, unsigned long long *out, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(out, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess || n <= 0) return e;
    count_launch();
    count_negative_kernel<<<blocks_for(n, 256), 256, 0, s>>>(p, n, out);
    return cudaGetLastError();
}

namespace {
__global__ void isolate_kernel(uint8_t *mat, void *J, int fp64, int nx, int ny, int nz, unsigned long long *n_ablated)
{
    const int64_t sy = nx, sz = (int64_t)nx * ny, n = sz * nz;
    GRID_STRIDE(v, n)
    {
        if (mat[v] == 0) continue;
        const int x = (int)(v % nx), y = (int)((v / nx) % ny), z = (int)(v / sz);
        // a neighbour outside the grid counts as air, as the reference's zero halo
        const bool air = (x == 0 || mat[v - 1] == 0) && (x == nx - 1 || mat[v + 1] == 0) &&
                         (y == 0 || mat[v - sy] == 0) && (y == ny - 1 || mat[v + sy] == 0) &&
                         (z == 0 || mat[v - sz] == 0) && (z == nz - 1 || mat[v + sz] == 0);
        if (air) {
            mat[v] = 0;
            if (fp64) ((double *)J)[v] = 0.0;
            else ((float *)J)[v] = 0.f;
            atomicAdd(n_ablated, 1ull);
        }
    }
}
}  // namespace

cudaError_t launch_isolate(uint8_t *mat, void *J, bool fp64, int nx, int ny, int nz, unsigned long long *n_ablated,
                           cudaStream_t s)
{
    const int64_t n = (int64_t)nx * ny * nz;
    if (n <= 0) return cudaSuccess;
    count_launch();
    isolate_kernel<<<blocks_for(n, 256), 256, 0, s>>>(mat, J, fp64 ? 1 : 0, nx, ny, nz, n_ablated);
    return cudaGetLastError();
}

}  // namespace tam
