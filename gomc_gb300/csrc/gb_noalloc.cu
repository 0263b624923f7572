// Reciprocal-space energy of caller-owned structure factors without any
// device allocation.
//
// Who needs this: a caller that may not allocate device memory once it is
// running -- a serving loop that admits jobs by device memory and has
// committed all of it to resident job state, or a host application whose
// device memory is owned by another allocator (a framework's caching
// allocator, a pool sized at start-up), where a cudaMalloc issued from inside
// this library would fail or fragment memory the host accounts for.  The box
// entry points (gb_box_reciprocal and the rest) grow per-box scratch on
// demand; this entry point never does.
//
// Scratch: one FP64 partial sum per 256 k-vectors lives in a file-scope
// device array of GB_RECIP_NOALLOC_MAX_PARTIALS doubles (8 KiB), so K is
// limited to GB_RECIP_NOALLOC_MAX_K.  Every partial is written before it is
// read, so nothing has to start at zero.  The device address of the array is
// looked up once per device, with that device current, on the first call
// made on it; that first call should come before any stream capture.  Calls
// that overlap in time on one device (two streams, two host threads) share
// the one array and race: serialise them.
//
// The summation order is the one of the box path (one partial per 256
// consecutive k-vectors, partials added in index order), so the result
// equals gb_box_reciprocal's on the same structure factors.
#include <mutex>

#include "gomc_gb300.h"
#include "gb_box.h"
#include "gb_pair.cuh"

namespace gb {

void set_api_error(const char *msg);

namespace {

constexpr int NT = 256;  // k-vectors per partial, threads per CTA
constexpr int MAX_DEVICES = 64;

static __device__ __align__(256) double
    g_recip_scratch[GB_RECIP_NOALLOC_MAX_PARTIALS];

std::mutex g_mutex;
double *g_scratch_ptr[MAX_DEVICES] = {};

__global__ void __launch_bounds__(NT)
    k_recip_energy_partials(int K, const double *__restrict__ sR,
                            const double *__restrict__ sI,
                            const double *__restrict__ prefact, double *part) {
  int k = blockIdx.x * NT + threadIdx.x;
  double e = 0.0;
  if (k < K)
    e = ((sR[k] * sR[k] + sI[k] * sI[k]) * prefact[k]);
  __shared__ double red[NT / 32];
  double s = block_sum<NT>(e, red);
  if (threadIdx.x == 0)
    part[blockIdx.x] = s;
}

__global__ void __launch_bounds__(NT)
    k_recip_energy_total(const double *__restrict__ part, int n, double *out) {
  __shared__ double red[NT / 32];
  double v = 0.0;
  for (int i = threadIdx.x; i < n; i += NT)
    v += part[i];
  double s = block_sum<NT>(v, red);
  if (threadIdx.x == 0)
    out[0] = s;
}

// Device address of the scratch array on the current device (looked up on
// the first call per device).
int scratch_for_current_device(double **out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    set_api_error(cudaGetErrorString(e));
    return ERR_CUDA;
  }
  if (dev < 0 || dev >= MAX_DEVICES) {
    set_api_error("device ordinal out of range");
    return ERR_ARG;
  }
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_scratch_ptr[dev]) {
    double *p = nullptr;
    e = cudaGetSymbolAddress((void **)&p, g_recip_scratch);
    if (e != cudaSuccess || !p) {
      set_api_error(e != cudaSuccess ? cudaGetErrorString(e)
                                     : "scratch symbol has no address");
      return ERR_CUDA;
    }
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return OK;
}

}  // namespace
}  // namespace gb

extern "C" int gb_recip_energy_noalloc(const double *d_sumR,
                                       const double *d_sumI,
                                       const double *d_prefact, int32_t K,
                                       double *d_energy, void *stream) {
  if (!d_energy || K < 0 || (K > 0 && (!d_sumR || !d_sumI || !d_prefact))) {
    gb::set_api_error("gb_recip_energy_noalloc: null pointer or negative K");
    return gb::ERR_ARG;
  }
  if (K > GB_RECIP_NOALLOC_MAX_K) {
    gb::set_api_error(
        "gb_recip_energy_noalloc: K exceeds GB_RECIP_NOALLOC_MAX_K "
        "(the fixed scratch holds one partial per 256 k-vectors)");
    return gb::ERR_CAPACITY;
  }
  double *scratch = nullptr;
  int rc = gb::scratch_for_current_device(&scratch);
  if (rc)
    return rc;
  cudaStream_t st = (cudaStream_t)stream;
  int nb = (K + gb::NT - 1) / gb::NT;
  if (nb > 0)
    gb::k_recip_energy_partials<<<nb, gb::NT, 0, st>>>(K, d_sumR, d_sumI,
                                                       d_prefact, scratch);
  gb::k_recip_energy_total<<<1, gb::NT, 0, st>>>(scratch, nb, d_energy);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    gb::set_api_error(cudaGetErrorString(e));
    return gb::ERR_CUDA;
  }
  return gb::OK;
}
