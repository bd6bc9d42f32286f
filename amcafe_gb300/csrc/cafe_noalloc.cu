// Allocation-free grain renumbering (the CleanLayer operation) on
// caller-owned device buffers.
//
// cafe_sim_clean_layer() allocates and frees its temporaries. Some callers
// cannot allow that: a host time loop that owns all device memory through its
// own pool and must not go back to the CUDA allocator after start-up, or one
// that must not incur the device-wide synchronisation that cudaFree implies
// while other work is in flight on its streams. For them,
// cafe_clean_layer_noalloc() performs the same renumbering on device arrays
// the caller already owns, and keeps its scratch in one fixed-size array that
// lives in this file for the life of the process.
//
// The scratch array below is held by every GPU that loads the library, until
// the process exits. It is shared by all calls: two calls whose work overlaps
// on the GPU (on different streams, or from different host threads) race on it
// and produce garbage; the caller must serialise them. Counters that must
// start at zero are cleared at the start of every call.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "../../include/cafe_gpu.h"

// Largest grain count a call accepts; the scratch holds, per grain, a volume
// count (int32), the new grain number (int32) and the compacted orientation
// (4 doubles), plus two int32 words: the new grain count and an input-error
// flag (set when a cell holds a grain ID outside 0..ngrain).
#define NOALLOC_SCRATCH_INTS (2 * CAFE_NOALLOC_MAX_GRAINS + 64)
#define NOALLOC_SCRATCH_BYTES (NOALLOC_SCRATCH_INTS * 4 + 4 * 8 * (size_t)CAFE_NOALLOC_MAX_GRAINS)

static __device__ __align__(256) unsigned char cafe_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

void cafe_internal_set_error(const char *msg);  // defined in cafe_host.cu

namespace {

const int kMaxDevices = 64;
void *g_scratch_addr[kMaxDevices] = {nullptr};
std::mutex g_scratch_mu;

struct ScratchView {
  int32_t *count;   // [CAFE_NOALLOC_MAX_GRAINS] cells per grain
  int32_t *newid;   // [CAFE_NOALLOC_MAX_GRAINS] new 1-based number, 0 = dropped
  int32_t *nnew;    // [2] grains kept, then the input-error flag
  int32_t *bad;     // == nnew + 1
  double *cth;      // [4 * CAFE_NOALLOC_MAX_GRAINS] compacted orientations
};

ScratchView view_of(void *base) {
  ScratchView v;
  int32_t *ip = (int32_t *)base;
  v.count = ip;
  v.newid = ip + CAFE_NOALLOC_MAX_GRAINS;
  v.nnew = ip + 2 * CAFE_NOALLOC_MAX_GRAINS;
  v.bad = v.nnew + 1;
  v.cth = (double *)((unsigned char *)base + (size_t)NOALLOC_SCRATCH_INTS * 4);
  return v;
}

// The caller's gid[] is not trusted: a grain ID outside 0..ngrain would index
// outside the caller's grain table (and past the scratch), so such a cell is
// skipped and the call's error flag is raised; the later kernels then change
// nothing.
__global__ void na_count(const int32_t *gid, long long ncell, int ngrain, int32_t *count, int32_t *bad) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ncell;
       i += (long long)gridDim.x * blockDim.x) {
    int g = gid[i];
    if (g > 0 && g <= ngrain)
      atomicAdd(&count[g - 1], 1);
    else if (g != 0)
      *bad = 1;
  }
}

// One block: grains with cells keep their order and are renumbered 1..k;
// their orientations are packed into the scratch.
__global__ void na_renumber(const int32_t *count, int32_t *newid, int32_t *nnew, const int32_t *bad,
                            const double *cth_in, double *cth_out, int ngrain) {
  __shared__ int part[1024];
  if (*bad) return;
  int per = (ngrain + blockDim.x - 1) / blockDim.x;
  int b0 = threadIdx.x * per, b1 = min(b0 + per, ngrain);
  int s = 0;
  for (int g = b0; g < b1; ++g) s += count[g] > 0;
  part[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int acc = 0;
    for (int t = 0; t < (int)blockDim.x; ++t) {
      int v = part[t];
      part[t] = acc;
      acc += v;
    }
    *nnew = acc;
  }
  __syncthreads();
  int k = part[threadIdx.x];
  for (int g = b0; g < b1; ++g) {
    if (count[g] > 0) {
      newid[g] = k + 1;
      for (int a = 0; a < 4; ++a) cth_out[4LL * k + a] = cth_in[4LL * g + a];
      ++k;
    } else {
      newid[g] = 0;
    }
  }
}

__global__ void na_remap(int32_t *gid, long long ncell, int ngrain, const int32_t *newid, const int32_t *bad) {
  if (*bad) return;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ncell;
       i += (long long)gridDim.x * blockDim.x) {
    int g = gid[i];
    if (g > 0 && g <= ngrain) gid[i] = newid[g - 1];
  }
}

__global__ void na_copy_back(const int32_t *nnew, const int32_t *bad, const double *cth_in, double *cth_out) {
  if (*bad) return;
  long long n = 4LL * *nnew;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    cth_out[i] = cth_in[i];
}

}  // namespace

extern "C" int cafe_clean_layer_noalloc(int32_t *gid, long long ncell, double *ctheta, int ngrain,
                                        int *ngrain_out, void *stream) {
  if (!gid || !ctheta || !ngrain_out || ncell < 0 || ngrain < 0) {
    cafe_internal_set_error("cafe_clean_layer_noalloc: null pointer or negative size");
    return CAFE_E_ARG;
  }
  if (ngrain > CAFE_NOALLOC_MAX_GRAINS) {
    cafe_internal_set_error("cafe_clean_layer_noalloc: ngrain exceeds CAFE_NOALLOC_MAX_GRAINS "
                            "(the fixed scratch size); use cafe_sim_clean_layer for larger grain tables");
    return CAFE_E_CAPACITY;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cafe_internal_set_error("cafe_clean_layer_noalloc: no usable current CUDA device");
    return CAFE_E_CUDA;
  }
  void *base = nullptr;
  {
    // First call on this device: look up the device address of the scratch
    // array with this device current (the host-side symbol is not a device
    // address and must never be handed to a kernel).
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
      void *p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, cafe_noalloc_scratch);
      if (e != cudaSuccess || !p) {
        cafe_internal_set_error("cafe_clean_layer_noalloc: cudaGetSymbolAddress failed");
        return CAFE_E_CUDA;
      }
      g_scratch_addr[dev] = p;
    }
    base = g_scratch_addr[dev];
  }
  cudaStream_t st = (cudaStream_t)stream;
  ScratchView v = view_of(base);
  int nsm = 1;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  int blocks = nsm * 8;
  // an error left by the caller's own earlier work is not this call's failure
  (void)cudaGetLastError();
  if (ngrain > 0) {
    if (cudaMemsetAsync(v.count, 0, (size_t)ngrain * sizeof(int32_t), st) != cudaSuccess) {
      cafe_internal_set_error("cafe_clean_layer_noalloc: clearing the scratch failed");
      return CAFE_E_CUDA;
    }
  }
  // the grain count and the input-error flag start at zero
  if (cudaMemsetAsync(v.nnew, 0, 2 * sizeof(int32_t), st) != cudaSuccess) {
    cafe_internal_set_error("cafe_clean_layer_noalloc: clearing the scratch failed");
    return CAFE_E_CUDA;
  }
  cudaError_t e = cudaSuccess;
  if (ngrain > 0) {
    na_count<<<blocks, 256, 0, st>>>(gid, ncell, ngrain, v.count, v.bad);
    e = cudaGetLastError();
    if (e == cudaSuccess) {
      na_renumber<<<1, 1024, 0, st>>>(v.count, v.newid, v.nnew, v.bad, ctheta, v.cth, ngrain);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
      na_remap<<<blocks, 256, 0, st>>>(gid, ncell, ngrain, v.newid, v.bad);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
      na_copy_back<<<blocks, 256, 0, st>>>(v.nnew, v.bad, v.cth, ctheta);
      e = cudaGetLastError();
    }
  } else if (ncell > 0) {
    // no grain table: every cell must be 0
    na_count<<<blocks, 256, 0, st>>>(gid, ncell, 0, v.count, v.bad);
    e = cudaGetLastError();
  }
  int32_t res[2] = {0, 0};
  if (e == cudaSuccess) e = cudaMemcpyAsync(res, v.nnew, sizeof(res), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    cafe_internal_set_error(cudaGetErrorString(e));
    return CAFE_E_CUDA;
  }
  if (res[1]) {
    cafe_internal_set_error("cafe_clean_layer_noalloc: gid holds a grain ID outside 0..ngrain; "
                            "gid and ctheta were left unchanged");
    return CAFE_E_ARG;
  }
  *ngrain_out = res[0];
  return CAFE_OK;
}
