// Per-box kinetic energy of atoms held in the caller's own device arrays,
// computed without any device allocation.
//
// Who needs it: a host MD code that keeps its atoms in device arrays it owns
// (CUDA Fortran or OpenACC data regions, or a pool allocator that reserved the
// free HBM when the run started) and wants the thermostat's per-box kinetic
// energy between its own kernels.  Such a caller cannot let a library allocate
// between steps.  A cudaMalloc there can fail or fragment the caller's pool,
// and cudaFree synchronises the whole device, which stalls the caller's other
// streams.  The context API allocates its arrays in examd_gpu_create.  This
// entry point reads the caller's velocity arrays in place and takes its
// scratch from one fixed file-scope device array instead.
//
// It is a variant of the context's kinetic-energy path: k_kinetic fills a
// per-atom energy buffer, then k_reduce_atoms (step.cu, used unchanged) sums it
// per box in a fixed order.  Here the per-atom buffer, the per-box sums, the
// box offsets and a status word all live in g_static_scratch.
//
// Limits and sharing:
//   * at most EXAMD_STATIC_MAX_ATOMS atoms and EXAMD_STATIC_MAX_BOXES boxes per
//     call; larger calls are rejected with EXAMD_ERR_ARG before any device work;
//   * every call on a device uses the same array, so two calls whose work
//     overlaps on that GPU (different host threads, or different streams with
//     no ordering between them) race and give wrong sums.  Calls issued one
//     after another from a single thread are safe: each call synchronises its
//     stream before it returns;
//   * the first call on a device resolves the array's address with
//     cudaGetSymbolAddress (this loads the module).  Make that first call
//     before any stream capture begins.  The address is cached for the life
//     of the process: a cudaDeviceReset of that device unloads the module and
//     leaves the cached address stale, so this entry point must not be used
//     on a device after the caller resets it.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/examd_gb300.h"
#include "kernels.cuh"

namespace {

constexpr int64_t kMaxAtoms = EXAMD_STATIC_MAX_ATOMS;
constexpr int kMaxBoxes = EXAMD_STATIC_MAX_BOXES;
constexpr int kMaxDevices = 64;

// Word offsets of the regions inside g_static_scratch (8-byte words).
constexpr size_t kOffKe = 0;                              // per-atom energy, kMaxAtoms doubles
constexpr size_t kOffBox = kOffKe + kMaxAtoms;            // per-box sums, kMaxBoxes doubles
constexpr size_t kOffAtom0 = kOffBox + kMaxBoxes;         // box offsets, kMaxBoxes + 1 int64
constexpr size_t kOffStatus = kOffAtom0 + kMaxBoxes + 1;  // status word (must start at zero)
constexpr size_t kWords = kOffStatus + 1;

struct Mass4 {
  double m[EXAMD_MAX_TYPES];
};

}  // namespace

// One instance per device (about 8.1 MB with the limits above).
static __device__ __align__(256) unsigned long long g_static_scratch[kWords];

namespace {

std::mutex g_setup_mu;
void* g_scratch_addr[kMaxDevices] = {};

// Same per-atom expression as k_kinetic; an out-of-range type sets bit 0 of
// the status word and contributes with the mass of type 0.
__global__ void k_kinetic_static(int64_t n, const double* __restrict__ vx, const double* __restrict__ vy,
                                 const double* __restrict__ vz, const int* __restrict__ type, int ntypes,
                                 const Mass4 mass, double* __restrict__ keAtom, unsigned int* status) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n) return;
  int t = type ? type[s] : 0;
  if ((unsigned)t >= (unsigned)ntypes) {
    atomicOr(status, 1u);
    t = 0;
  }
  keAtom[s] = 0.5 * mass.m[t] * (vx[s] * vx[s] + vy[s] * vy[s] + vz[s] * vz[s]);
}

void put_err(char* buf, int len, const char* msg) {
  if (buf && len > 0) {
    std::strncpy(buf, msg, (size_t)len - 1);
    buf[len - 1] = '\0';
  }
}

// The caller's arrays must be device (or managed) memory of this device: a
// host pointer handed to the kernel would fault the GPU instead of failing.
bool device_readable(const void* p, int dev) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (a.type == cudaMemoryTypeManaged) return true;
  return a.type == cudaMemoryTypeDevice && a.device == dev;
}

}  // namespace

extern "C" int examd_kinetic_static(int device, int64_t natoms, int nboxes, const int64_t* atom0,
                                    const double* vx, const double* vy, const double* vz, const int* type,
                                    int ntypes, const double* mass, double* ekin, void* stream, char* errbuf,
                                    int errbuf_len) {
  char msg[192];
  put_err(errbuf, errbuf_len, "");
  // Host-side checks first: an oversized call is rejected before any CUDA call.
  if (natoms < 0 || natoms > kMaxAtoms) {
    std::snprintf(msg, sizeof msg, "natoms %lld outside [0, %lld] (the static scratch limit)", (long long)natoms,
                  (long long)kMaxAtoms);
    put_err(errbuf, errbuf_len, msg);
    return EXAMD_ERR_ARG;
  }
  if (nboxes < 1 || nboxes > kMaxBoxes) {
    std::snprintf(msg, sizeof msg, "nboxes %d outside [1, %d] (the static scratch limit)", nboxes, kMaxBoxes);
    put_err(errbuf, errbuf_len, msg);
    return EXAMD_ERR_ARG;
  }
  if (!atom0 || !ekin || !mass || ntypes < 1 || ntypes > EXAMD_MAX_TYPES || (natoms > 0 && (!vx || !vy || !vz))) {
    put_err(errbuf, errbuf_len, "NULL array, or ntypes outside [1, 4]");
    return EXAMD_ERR_ARG;
  }
  if (atom0[0] != 0 || atom0[nboxes] != natoms) {
    put_err(errbuf, errbuf_len, "atom0 must start at 0 and end at natoms");
    return EXAMD_ERR_ARG;
  }
  for (int b = 0; b < nboxes; ++b)
    if (atom0[b + 1] < atom0[b]) {
      put_err(errbuf, errbuf_len, "atom0 must be nondecreasing");
      return EXAMD_ERR_ARG;
    }
  Mass4 m4{};
  for (int t = 0; t < ntypes; ++t) {
    if (!(std::isfinite(mass[t]) && mass[t] > 0.0)) {
      put_err(errbuf, errbuf_len, "masses must be finite and positive");
      return EXAMD_ERR_ARG;
    }
    m4.m[t] = mass[t];
  }

  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    put_err(errbuf, errbuf_len, "no CUDA device");
    return EXAMD_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= ndev || device >= kMaxDevices) {
    put_err(errbuf, errbuf_len, "device index out of range");
    return EXAMD_ERR_ARG;
  }
  int prev = -1;
  cudaGetDevice(&prev);
  if (cudaSetDevice(device) != cudaSuccess) {
    cudaGetLastError();
    put_err(errbuf, errbuf_len, "cudaSetDevice failed");
    return EXAMD_ERR_CUDA;
  }
  int rc = EXAMD_OK;
  auto fail = [&](int code, const char* what, cudaError_t e) {
    std::snprintf(msg, sizeof msg, "%s: %s", what, cudaGetErrorString(e));
    put_err(errbuf, errbuf_len, msg);
    rc = code;
  };

  // Set-up, once per device with that device current.
  unsigned long long* base = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_addr[device]) {
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
      if (e != cudaSuccess || !p) {
        fail(EXAMD_ERR_CUDA, "cudaGetSymbolAddress", e);
        cudaSetDevice(prev >= 0 ? prev : device);
        return rc;
      }
      g_scratch_addr[device] = p;
    }
    base = static_cast<unsigned long long*>(g_scratch_addr[device]);
  }

  if (natoms > 0 && !(device_readable(vx, device) && device_readable(vy, device) && device_readable(vz, device) &&
                      (!type || device_readable(type, device)))) {
    put_err(errbuf, errbuf_len, "vx, vy, vz and type must be device memory of the given device");
    cudaSetDevice(prev >= 0 ? prev : device);
    return EXAMD_ERR_ARG;
  }

  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double* keAtom = reinterpret_cast<double*>(base + kOffKe);
  double* boxKE = reinterpret_cast<double*>(base + kOffBox);
  int64_t* d_atom0 = reinterpret_cast<int64_t*>(base + kOffAtom0);
  unsigned int* status = reinterpret_cast<unsigned int*>(base + kOffStatus);
  unsigned int h_status = 0;
  cudaError_t e;
  if ((e = cudaMemsetAsync(status, 0, sizeof(unsigned int), st)) != cudaSuccess) {
    fail(EXAMD_ERR_CUDA, "clearing the status word", e);
  } else if ((e = cudaMemcpyAsync(d_atom0, atom0, (nboxes + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, st)) !=
             cudaSuccess) {
    fail(EXAMD_ERR_CUDA, "copying atom0", e);
  } else {
    if (natoms > 0)
      k_kinetic_static<<<(unsigned)((natoms + 255) / 256), 256, 0, st>>>(natoms, vx, vy, vz, type, ntypes, m4,
                                                                         keAtom, status);
    if ((e = cudaGetLastError()) != cudaSuccess) {
      fail(EXAMD_ERR_CUDA, "k_kinetic_static launch", e);
    } else if ((e = examd::launch_reduce_atoms(nboxes, d_atom0, keAtom, boxKE, st)) != cudaSuccess) {
      fail(EXAMD_ERR_CUDA, "k_reduce_atoms launch", e);
    } else if ((e = cudaMemcpyAsync(ekin, boxKE, nboxes * sizeof(double), cudaMemcpyDeviceToHost, st)) !=
                   cudaSuccess ||
               (e = cudaMemcpyAsync(&h_status, status, sizeof(unsigned int), cudaMemcpyDeviceToHost, st)) !=
                   cudaSuccess ||
               (e = cudaStreamSynchronize(st)) != cudaSuccess) {
      fail(EXAMD_ERR_CUDA, "reading the result", e);
    } else if (h_status) {
      put_err(errbuf, errbuf_len, "a type index is outside [0, ntypes)");
      rc = EXAMD_ERR_ARG;
    }
  }
  // On a failure after work was queued, wait for that work before returning,
  // so that no kernel or copy of this call still touches the shared array when
  // the next call (perhaps on another stream) starts.  The wait's own result
  // is ignored: the status already reports the first failure.
  if (rc != EXAMD_OK) {
    cudaStreamSynchronize(st);
    cudaGetLastError();
  }
  cudaSetDevice(prev >= 0 ? prev : device);
  return rc;
}
