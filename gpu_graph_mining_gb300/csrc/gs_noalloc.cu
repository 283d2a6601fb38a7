// Support counting that allocates no memory, for callers that may not call
// cudaMalloc: code that runs inside another framework's memory arena or
// allocator (which owns every device allocation and accounts for it), hosts
// with a fixed device-memory budget handed out up front, and code paths that
// must not trigger the implicit device synchronisation cudaMalloc/cudaFree can
// cause.  The caller passes device buffers it already owns for the inputs and
// the output; the only scratch, the support bitmaps, lives in the file-scope
// device array below, which every GPU that loads this library holds until the
// process exits.
//
// Same result as gs_support_count (support[k] = number of distinct graph ids
// among the records whose key is k), computed by the same three steps:
// clear the bitmap, set bit [key][graph] per record, popcount per key.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "../../include/gspan_gb300.h"

namespace {

constexpr unsigned kScratchWords = GS_NOALLOC_MAX_BITMAP_WORDS;  // 4 MiB
constexpr int kMaxDevices = 64;
constexpr int kBlock = 256;

// The scratch shared by every call on a device.
static __device__ __align__(256) uint32_t g_noalloc_bitmap[kScratchWords];

std::mutex g_mu;

}  // namespace

namespace gsgb {
// the library's thread-local error text (gs_last_error), kept in gs_capi.cpp
void capi_set_error(const char *msg);
}  // namespace gsgb

namespace {

struct ErrText {
  void operator=(const char *m) { gsgb::capi_set_error(m); }
} t_msg;

__global__ void k_clear(uint32_t *bm, long long words)
{
  const long long stride = (long long)gridDim.x * blockDim.x;
  for(long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < words; i += stride) bm[i] = 0u;
}

// Records outside [0, n_keys) x [0, n_graphs) are skipped.
__global__ void k_mark(uint32_t *bm, const int32_t *__restrict__ keys, const int32_t *__restrict__ gids, long long n,
                       int n_keys, int n_graphs, int words)
{
  const long long stride = (long long)gridDim.x * blockDim.x;
  for(long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int k = keys[i], g = gids[i];
    if((unsigned)k >= (unsigned)n_keys || (unsigned)g >= (unsigned)n_graphs) continue;
    atomicOr(&bm[(long long)k * words + (g >> 5)], 1u << (g & 31));
  }
}

// One warp per key.
__global__ void k_count(const uint32_t *__restrict__ bm, int n_keys, int words, int32_t *support)
{
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for(int key = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; key < n_keys; key += warps) {
    int c = 0;
    for(int w = lane; w < words; w += 32) c += __popc(bm[(long long)key * words + w]);
    for(int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if(lane == 0) support[key] = c;
  }
}

// Per device: the scratch's device address and the SM count, looked up once.
struct DevInfo {
  uint32_t *addr = nullptr;
  int sms = 0;
};
DevInfo g_dev[kMaxDevices];

int grid_for(long long n, int sms)
{
  long long b = (n + kBlock - 1) / kBlock;
  if(b < 1) b = 1;
  const long long cap = 8LL * sms;  // 8 blocks of 256 threads per SM, grid-stride beyond
  return (int)(b < cap ? b : cap);
}

// Restores the calling thread's current device on every return path.
struct CurrentDevice {
  int prev = -1;
  bool changed = false;
  bool set(int dev)
  {
    if(cudaGetDevice(&prev) != cudaSuccess) {
      cudaGetLastError();
      prev = -1;
    }
    if(prev == dev) return true;
    if(cudaSetDevice(dev) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    changed = prev >= 0;
    return true;
  }
  ~CurrentDevice()
  {
    if(changed) cudaSetDevice(prev);
  }
};

// The device that owns `p` (device or managed memory), or -1.
int device_of(const void *p)
{
  cudaPointerAttributes a;
  if(cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return -1;
  }
  if(a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged) return -1;
  return a.device;
}

// Scratch address and SM count of device `dev`, which must be current.  The
// first call per device resolves the address with cudaGetSymbolAddress
// (which may load the module) and caches it for the life of the process.
gs_status device_info(int dev, DevInfo *out)
{
  if(dev < 0 || dev >= kMaxDevices) {
    t_msg = "gs_support_count_noalloc: device index out of range";
    return GS_ERR_LIMIT;
  }
  std::lock_guard<std::mutex> g(g_mu);
  DevInfo &d = g_dev[dev];
  if(!d.addr) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_bitmap);
    int sms = 0;
    if(e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if(e != cudaSuccess || !p || sms <= 0) {
      cudaGetLastError();
      t_msg = "gs_support_count_noalloc: cudaGetSymbolAddress of the scratch failed";
      return GS_ERR_CUDA;
    }
    d.sms = sms;
    d.addr = (uint32_t *)p;
  }
  *out = d;
  return GS_OK;
}

}  // namespace

extern "C" gs_status gs_support_count_noalloc(const int32_t *d_keys, const int32_t *d_graph_ids, int64_t n_records,
                                              int32_t n_keys, int32_t n_graphs, int32_t *d_support, void *stream)
{
  t_msg = "";
  if(n_records < 0 || n_keys < 0 || n_graphs < 0 || (n_records > 0 && (!d_keys || !d_graph_ids)) ||
     (n_keys > 0 && !d_support)) {
    t_msg = "gs_support_count_noalloc: invalid arguments";
    return GS_ERR_USAGE;
  }
  if(n_keys == 0) return GS_OK;
  const long long words = n_graphs > 0 ? ((long long)n_graphs + 31) / 32 : 1;
  if((long long)n_keys * words > (long long)kScratchWords) {
    t_msg = "gs_support_count_noalloc: n_keys * ceil(n_graphs/32) exceeds the 1048576-word (4 MiB) scratch";
    return GS_ERR_LIMIT;
  }
  // The work runs on the device that holds d_support; the stream must belong to it.
  const int dev = device_of(d_support);
  if(dev < 0) {
    t_msg = "gs_support_count_noalloc: d_support is not device memory";
    return GS_ERR_USAGE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  CurrentDevice cur;
  if(!cur.set(dev)) {
    t_msg = "gs_support_count_noalloc: cannot make the device of d_support current";
    return GS_ERR_CUDA;
  }
  if(s) {
    int sdev = -1;
    if(cudaStreamGetDevice(s, &sdev) != cudaSuccess) {
      cudaGetLastError();
      t_msg = "gs_support_count_noalloc: invalid stream";
      return GS_ERR_USAGE;
    }
    if(sdev != dev) {
      t_msg = "gs_support_count_noalloc: the stream belongs to another device than d_support";
      return GS_ERR_USAGE;
    }
  }
  // An error left pending by the caller's earlier work is reported as such
  // and left in place (peek, not get), so a launch error below is this call's.
  const cudaError_t pending = cudaPeekAtLastError();
  if(pending != cudaSuccess) {
    t_msg = "gs_support_count_noalloc: an earlier CUDA error is pending; nothing was launched";
    return GS_ERR_CUDA;
  }
  DevInfo di;
  gs_status st = device_info(dev, &di);
  if(st != GS_OK) return st;
  uint32_t *bm = di.addr;
  const long long nw = (long long)n_keys * words;
  k_clear<<<grid_for(nw, di.sms), kBlock, 0, s>>>(bm, nw);
  if(cudaGetLastError() != cudaSuccess) {
    t_msg = "gs_support_count_noalloc: launch of the scratch clear failed";
    return GS_ERR_CUDA;
  }
  if(n_records > 0) {
    k_mark<<<grid_for(n_records, di.sms), kBlock, 0, s>>>(bm, d_keys, d_graph_ids, n_records, n_keys, n_graphs,
                                                          (int)words);
    if(cudaGetLastError() != cudaSuccess) {
      t_msg = "gs_support_count_noalloc: launch of the record marking failed";
      return GS_ERR_CUDA;
    }
  }
  k_count<<<grid_for((long long)n_keys * 32, di.sms), kBlock, 0, s>>>(bm, n_keys, (int)words, d_support);
  if(cudaGetLastError() != cudaSuccess) {
    t_msg = "gs_support_count_noalloc: launch of the popcount failed";
    return GS_ERR_CUDA;
  }
  return GS_OK;
}
