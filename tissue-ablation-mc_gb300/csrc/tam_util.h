// tam_util.h -- launchers of the set-up / conversion kernels (util.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace tam {

// Per-material lookup table passed by value to the conversion kernels.
struct MatThermal {
    double k[16], rho[16], c[16], mut[16];
};

cudaError_t launch_fill_f64(double *p, double v, int64_t n, cudaStream_t s);
cudaError_t launch_fill_real(void *p, bool fp64, double v, int64_t n, cudaStream_t s);
cudaError_t launch_fill_u8(uint8_t *p, uint8_t v, int64_t n, cudaStream_t s);
cudaError_t launch_fill_halo(double *p, int nx, int ny, int nz, double vin, double vhalo, double vtop, bool has_top,
                             cudaStream_t s);
cudaError_t launch_ref_init_temp(double *p, int nx, int ny, int nz, cudaStream_t s);
cudaError_t launch_props_from_mat(const uint8_t *mat, int nmat, const MatThermal &lut, void *k, void *r, void *c,
                                  bool fp64, int64_t n, cudaStream_t s);
cudaError_t launch_to_f64(const void *src, bool fp64, double *dst, int64_t n, cudaStream_t s);
cudaError_t launch_from_f64(const double *src, void *dst, bool fp64, int64_t n, cudaStream_t s);
cudaError_t launch_interior_to_halo(const void *src, bool fp64, double *halo, int nx, int ny, int nz, cudaStream_t s);
cudaError_t launch_halo_to_interior(const double *halo, void *dst, bool fp64, int nx, int ny, int nz, cudaStream_t s);
cudaError_t launch_rhokap_from_mat(const uint8_t *mat, int nmat, const MatThermal &lut, double *halo, int nx, int ny,
                                   int nz, cudaStream_t s);
cudaError_t launch_count_negative(const double *p, int64_t n, unsigned long long *out, cudaStream_t s);

}  // namespace tam
