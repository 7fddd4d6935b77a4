// noalloc.cu -- an MC pass that allocates no device memory.
//
// Some callers cannot call cudaMalloc: a Fortran host whose device arrays are
// owned by another runtime (OpenACC / CUDA Fortran) and that must not grow the
// device heap behind that runtime's back, or a host running under a fixed
// device-memory budget.  tam_mc_pass_noalloc serves them: the caller
// passes the input (rhokap) and output (jmeanGLOBAL) as device pointers, and
// the pass's scratch -- the FP64 tally in packet units, the escape tallies,
// the packet work counter and the device error word -- lives in the
// file-scope array below, which every GPU that loads this library holds until
// the process exits.  The call is synchronous: it reads the pass's error word
// back before it returns.
#include <atomic>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "../../include/tam.h"
#include "tam_kernels.h"

namespace {

// Layout of the scratch array (doubles): [0, 16) escape tallies,
// [16] packet work counter (as unsigned long long), [17] device error word
// (as unsigned), [32, 32 + nx*ny*nz) the per-voxel tally of the pass.
constexpr int64_t HEAD = 32;
constexpr int64_t SCRATCH_DOUBLES = HEAD + (int64_t)TAM_NOALLOC_MAX_VOXELS;

static __device__ __align__(256) double g_scratch[SCRATCH_DOUBLES];

constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
double *g_ptr[MAX_DEVICES] = {nullptr};  // device address of g_scratch, per device

int fail(int code, const std::string &m)
{
    tam::set_thread_error(m);  // reported by tam_last_error(NULL)
    return code;
}

// Device address of the scratch array on the current device.  The first call
// on a device looks it up (cudaGetSymbolAddress) and keeps it for the rest of
// the process, so a cudaDeviceReset of that device afterwards is not
// supported; the host-side symbol itself is only a stand-in and must never be
// handed to a kernel.
int scratch_on_current_device(double **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(TAM_E_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= MAX_DEVICES) return fail(TAM_E_INVALID, "device ordinal beyond the scratch table");
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess || !p)
            return fail(TAM_E_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
        g_ptr[dev] = (double *)p;
    }
    *out = g_ptr[dev];
    return TAM_OK;
}

}  // namespace

extern "C" int tam_mc_pass_noalloc(const tam_params *p, const double *rhokap, double *jmean_global, int64_t nphotons,
                                   uint64_t seed, uint32_t stream, double power, void *cuda_stream)
{
    if (!p || !rhokap || !jmean_global) return fail(TAM_E_INVALID, "null argument");
    if (p->nxg < 1 || p->nyg < 1 || p->nzg < 1 || !(p->xmax > 0) || !(p->ymax > 0) || !(p->zmax > 0))
        return fail(TAM_E_INVALID, "grid sizes and half-widths must be positive");
    if (nphotons < 0) return fail(TAM_E_INVALID, "nphotons must be >= 0");
    if (p->precision != TAM_FP64 && p->precision != TAM_FP32) return fail(TAM_E_INVALID, "bad precision");
    const int64_t ni = (int64_t)p->nxg * p->nyg * p->nzg;
    if (ni > (int64_t)TAM_NOALLOC_MAX_VOXELS)
        return fail(TAM_E_INVALID, "grid of " + std::to_string(ni) + " voxels exceeds the allocation-free limit of " +
                                       std::to_string((long long)TAM_NOALLOC_MAX_VOXELS) + " voxels");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        (void)cudaGetLastError();
        return fail(TAM_E_NODEV, "no CUDA device");
    }
    // the caller's runtime owns the choice of device: run on the current one,
    // which p->device must name, rather than switching devices behind its back
    int cur = -1;
    if (cudaGetDevice(&cur) != cudaSuccess) {
        (void)cudaGetLastError();
        return fail(TAM_E_CUDA, "cudaGetDevice failed");
    }
    if (p->device != cur)
        return fail(TAM_E_INVALID, "p->device (" + std::to_string(p->device) + ") is not the current device (" +
                                       std::to_string(cur) + ")");
    double *base = nullptr;
    int r = scratch_on_current_device(&base);
    if (r != TAM_OK) return r;
    cudaStream_t s = (cudaStream_t)cuda_stream;
    double *tally = base;
    unsigned long long *work = (unsigned long long *)(base + 16);
    unsigned *err = (unsigned *)(base + 17);
    double *acc = base + HEAD;
    // every call shares the scratch: clear what the pass accumulates into
    cudaError_t e = cudaMemsetAsync(base, 0, (size_t)(HEAD + ni) * sizeof(double), s);
    if (e != cudaSuccess) return fail(TAM_E_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));

    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, cur);
    // sourcephCO2 + tauint1 of the reference (pure absorber, uniform disk of
    // diameter 250 um, no Fresnel, no roulette), as tam_mc_pass in reference mode
    tam::TransportArgs a{};
    a.nx = p->nxg;
    a.ny = p->nyg;
    a.nz = p->nzg;
    a.xmax = p->xmax;
    a.ymax = p->ymax;
    a.zmax = p->zmax;
    a.medium = tam::MED_RHOKAP;
    a.rhokap = rhokap;
    a.rhokap_n = p->n2;
    a.n_ambient = p->n1;
    a.source = tam::SRC_DISK;
    a.source_radius = 250e-4 / 2.;
    a.fresnel = 0;
    a.roulette = 0;
    a.roulette_w = 0.0;
    a.roulette_m = 1.0;
    a.max_steps = (int64_t)1 << 40;
    a.nudge = 1.e-8 * (2. * p->zmax / p->nzg);  // src/mcpolar.f90:112
    a.scat_min = 0;
    a.uniform_id = -1;
    a.seed = seed;
    a.stream = stream;
    a.p0 = 0;
    a.n = nphotons;
    a.jmean = acc;
    a.tally = tally;
    a.work = work;
    a.err = err;
    e = tam::launch_transport(a, p->precision == TAM_FP64, sms, s);
    if (e != cudaSuccess) return fail(TAM_E_CUDA, std::string("transport: ") + cudaGetErrorString(e));
    // jmeanGLOBAL = jmean * (P/81) / (nphotons * Vvox)   (src/mcpolar.f90:174)
    const double den = (double)nphotons * (2. * p->xmax * 1.e-2 / p->nxg) * (2. * p->ymax * 1.e-2 / p->nyg) *
                       (2. * p->zmax * 1.e-2 / p->nzg);
    const double f = nphotons > 0 ? (power / 81.0) / den : 0.0;
    e = tam::launch_scale_f64(jmean_global, acc, f, ni, false, s);
    if (e != cudaSuccess) return fail(TAM_E_CUDA, std::string("normalise: ") + cudaGetErrorString(e));
    unsigned bits = 0;
    e = cudaMemcpyAsync(&bits, err, sizeof bits, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(TAM_E_CUDA, std::string("tam_mc_pass_noalloc: ") + cudaGetErrorString(e));
    if (bits) {
        char buf[64];
        std::snprintf(buf, sizeof buf, "device error word 0x%x", bits);
        return fail(TAM_E_DEVICE, buf);
    }
    return TAM_OK;
}
