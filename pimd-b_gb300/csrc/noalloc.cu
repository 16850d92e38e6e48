// Exchange evaluation that allocates nothing.
//
// Some callers cannot call cudaMalloc at the moment they need the bosonic
// exchange: a host program whose device memory is owned by another allocator
// or held to a fixed budget (a cudaMalloc behind its back would fail or break
// its accounting), or a latency-critical loop that must not pay the implicit
// device synchronisation of cudaMalloc/cudaFree.  pimdb_exchange_noalloc
// serves them: the caller passes device inputs and outputs, and every
// intermediate array of the exchange (cycle energies, weights, potentials,
// work flags) lives in one file-scope __device__ array of fixed size,
// reserved on every GPU that loads this library for as long as the process
// lives.
//
// The fixed size limits the system to kNoAllocMaxN particles.  Every call
// reuses the same array and leaves its contents behind, so each call first
// clears the flags that must start at zero, and two calls that overlap on the
// GPU (on different streams, or from different host threads) race on it.
// The first call on a device looks up the array's device address
// (cudaGetSymbolAddress, with that device current); make that first call
// before any stream capture.  The call synchronises `cuda_stream` and reads
// an error word back before it returns.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>
#include <string>

#include "../../include/pimdb_gb300.h"
#include "common.cuh"
#include "kernels.h"

namespace pimdb {

constexpr int kNoAllocMaxN = 256;
constexpr int kNoAllocLd = 256;  // particle stride (multiple of 32, >= kNoAllocMaxN)
constexpr size_t kTri = (size_t)kNoAllocMaxN * (kNoAllocMaxN + 1) / 2;
constexpr size_t kVec = kNoAllocMaxN + 1;
// layout, in doubles
constexpr size_t kOffX = 0;                              // 4 beads x 3 axes x ld
constexpr size_t kOffFx = kOffX + 4 * 3 * kNoAllocLd;    // 2 x 3 x ld
constexpr size_t kOffE = kOffFx + 2 * 3 * kNoAllocLd;
constexpr size_t kOffWf = kOffE + kTri;
constexpr size_t kOffWb = kOffWf + kTri;
constexpr size_t kOffEt = kOffWb + kTri;
constexpr size_t kOffV = kOffEt + kTri;                  // V, Vb, Vh, Vbh, yf, yb
constexpr size_t kOffRow = kOffV + 6 * kVec;             // rowR, rowC
constexpr size_t kOffScal = kOffRow + 2 * kNoAllocMaxN;  // 4 scalars
constexpr size_t kOffFlags = kOffScal + 4;               // 16 ints (8 doubles)
constexpr size_t kScratchDoubles = kOffFlags + 8;

// About 1.1 MB per GPU.
static __device__ __align__(256) double g_exchange_scratch[kScratchDoubles];

// Gathers beads 1, 2, P-1 and P of the caller's ring x[P][N][D] into the
// scratch layout (as beads 0..3 of a 4-bead ring, which is all the exchange
// reads) and clears the work flags.
__global__ void k_noalloc_prepare(Sys s, const double* __restrict__ ring, int P, int D) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e == 9) s.xflags[kExchRowsCount] = 0;  // the energy kernel's block count
    if (e < 8) {
        s.xflags[e] = (e == 3) ? 1 : 0;  // [3]: compute a fresh estimate
        if (e == 0) {
            *s.err = 0;
        }
    }
    const int n = s.N * D;
    if (e >= 4 * n) return;
    const int mb = e / n, rem = e % n, i = rem / D, a = rem % D;
    const int src_bead = mb == 0 ? 0 : (mb == 1 ? 1 % P : (mb == 2 ? (P - 2 + P) % P : P - 1));
    s.x[((size_t)mb * D + a) * s.ld + i] = ring[((size_t)src_bead * s.N + i) * D + a];
}

__global__ void k_noalloc_finish(Sys s, int D, double* scalars, double* f_first, double* f_last) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < 4 && scalars) scalars[e] = s.scal[e];
    if (e >= s.N * D) return;
    const int i = e / D, a = e % D;
    if (f_first) f_first[e] = s.fx[((size_t)0 * D + a) * s.ld + i];
    if (f_last) f_last[e] = s.fx[((size_t)1 * D + a) * s.ld + i];
}

}  // namespace pimdb

using namespace pimdb;

static std::mutex g_noalloc_mu;
static double* g_noalloc_ptr[128] = {};

extern "C" int pimdb_exchange_noalloc(const double* ring, int nbeads, int natoms, int ndim, double spring_constant,
                                      double beta_ex, int pbc, double box, double* scalars, double* f_first,
                                      double* f_last, void* cuda_stream, char* err, int err_len) {
    auto report = [&](const std::string& m) {
        if (err && err_len > 0) std::snprintf(err, (size_t)err_len, "%s", m.c_str());
    };
    report("");
    if (!ring) {
        report("ring coordinates missing");
        return PIMDB_ERR_ARG;
    }
    if (natoms < 1 || natoms > kNoAllocMaxN) {
        report("pimdb_exchange_noalloc handles 1.." + std::to_string(kNoAllocMaxN) + " particles, got " +
               std::to_string(natoms));
        return PIMDB_ERR_ARG;
    }
    if (ndim < 1 || ndim > 3 || nbeads < 2 || !(spring_constant > 0.0) || !(beta_ex > 0.0) || (pbc && !(box > 0.0))) {
        report("invalid ndim, nbeads (needs at least 2), spring constant, beta or box");
        return PIMDB_ERR_ARG;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 128) {
        cudaGetLastError();
        report("no usable CUDA device");
        return PIMDB_ERR_NO_DEVICE;
    }
    if (cuda_stream) {
        // the scratch address below is the current device's: the stream must
        // belong to that device
        int sdev = -1;
        if (cudaStreamGetDevice((cudaStream_t)cuda_stream, &sdev) != cudaSuccess) {
            cudaGetLastError();
            report("cuda_stream is not a valid CUDA stream");
            return PIMDB_ERR_ARG;
        }
        if (sdev != dev) {
            report("cuda_stream belongs to device " + std::to_string(sdev) + " but device " + std::to_string(dev) +
                   " is current");
            return PIMDB_ERR_ARG;
        }
    }
    double* base = nullptr;
    {
        // Once per device, with that device current: the array's name is only
        // a host-side stand-in, the kernels need its device address.
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        if (!g_noalloc_ptr[dev]) {
            const cudaError_t e = cudaGetSymbolAddress((void**)&g_noalloc_ptr[dev], g_exchange_scratch);
            if (e != cudaSuccess) {
                g_noalloc_ptr[dev] = nullptr;
                report(std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
                return PIMDB_ERR_CUDA;
            }
        }
        base = g_noalloc_ptr[dev];
    }
    cudaStream_t st = (cudaStream_t)cuda_stream;
    Sys s{};
    s.N = natoms;
    s.P = 4;  // the gathered beads 1, 2, P-1, P
    s.ld = kNoAllocLd;
    s.bosonic = 1;
    s.pbc = pbc ? 1 : 0;
    s.L = pbc ? box : 1.0;
    s.invL = 1.0 / s.L;
    s.kappa = spring_constant;
    s.beta_ex = beta_ex;
    s.inv_beta_ex = 1.0 / beta_ex;
    s.x = base + kOffX;
    s.fx = base + kOffFx;
    s.E = base + kOffE;
    s.Wf = base + kOffWf;
    s.Wb = base + kOffWb;
    s.Et = base + kOffEt;
    s.V = base + kOffV;
    s.Vb = s.V + kVec;
    s.Vh = s.V + 2 * kVec;
    s.Vbh = s.V + 3 * kVec;
    s.yf = s.V + 4 * kVec;
    s.yb = s.V + 5 * kVec;
    s.rowR = base + kOffRow;
    s.rowC = s.rowR + kNoAllocMaxN;
    s.scal = base + kOffScal;
    s.xflags = reinterpret_cast<int*>(base + kOffFlags);
    s.err = s.xflags + 8;
    const int n4 = 4 * natoms * ndim;
    k_noalloc_prepare<<<(n4 + 255) / 256, 256, 0, st>>>(s, ring, nbeads, ndim);
    const int est = launch_exchange_energies(s, ndim, st);
    launch_exchange_recursions(s, 0, st, nullptr, nullptr, est);
    launch_exchange_forces_mode(s, ndim, 0, st);
    Sys se = s;
    se.P = nbeads;  // primEstimator divides by the true number of beads
    launch_exchange_estimators(se, st);
    const int nf = natoms * ndim;
    k_noalloc_finish<<<(nf + 255) / 256 + 1, 256, 0, st>>>(s, ndim, scalars, f_first, f_last);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    int derr = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&derr, s.err, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        report(std::string("CUDA: ") + cudaGetErrorString(e));
        return PIMDB_ERR_CUDA;
    }
    if (derr & ERRB_NONFINITE_VB) {
        report("Invalid sig_denom in bosonic exchange potential");
        return PIMDB_ERR_NONFINITE_VB;
    }
    return PIMDB_OK;
}
