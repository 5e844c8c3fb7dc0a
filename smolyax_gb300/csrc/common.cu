// Error reporting and small utilities (scan) shared by the library.
#include "common.cuh"

namespace smx {

static thread_local std::string g_last_error;

int set_error(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    return set_error(SMX_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  }
  return SMX_OK;
}

}  // namespace smx

namespace {

constexpr int kScanBlock = 512;
constexpr int kScanItems = 4;  // items per thread
constexpr int64_t kScanTile = int64_t(kScanBlock) * kScanItems;

__device__ inline int64_t block_exclusive_scan(int64_t v, int64_t* sh, int64_t* total) {
  // Hillis-Steele over a warp, then over warp totals.
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int64_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[warp] = x;
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    int64_t w = lane < nw ? sh[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int64_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < nw) sh[lane] = w;
  }
  __syncthreads();
  int64_t warp_prefix = warp > 0 ? sh[warp - 1] : 0;
  *total = sh[(blockDim.x >> 5) - 1];
  __syncthreads();
  return warp_prefix + x - v;
}

__global__ void scan_tile_sums(const int64_t* __restrict__ in, int64_t n, int64_t* __restrict__ sums) {
  __shared__ int64_t sh[32];
  int64_t base = int64_t(blockIdx.x) * kScanTile;
  int64_t s = 0;
  for (int i = 0; i < kScanItems; ++i) {
    int64_t idx = base + int64_t(i) * kScanBlock + threadIdx.x;
    if (idx < n) s += in[idx];
  }
  int64_t tot;
  block_exclusive_scan(s, sh, &tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void scan_sums_serial(int64_t* sums, int64_t nt) {
  // single block: exclusive scan of the tile sums in chunks
  __shared__ int64_t sh[32];
  int64_t carry = 0;
  for (int64_t b0 = 0; b0 < nt; b0 += blockDim.x) {
    int64_t idx = b0 + threadIdx.x;
    int64_t v = idx < nt ? sums[idx] : 0;
    int64_t tot;
    int64_t ex = block_exclusive_scan(v, sh, &tot);
    if (idx < nt) sums[idx] = carry + ex;
    carry += tot;
  }
  if (threadIdx.x == 0) sums[nt] = carry;
}

__global__ void scan_tiles(const int64_t* __restrict__ in, int64_t* __restrict__ out, int64_t n,
                           const int64_t* __restrict__ sums) {
  __shared__ int64_t sh[32];
  int64_t base = int64_t(blockIdx.x) * kScanTile + int64_t(threadIdx.x) * kScanItems;
  int64_t v[kScanItems];
  int64_t s = 0;
  for (int i = 0; i < kScanItems; ++i) {
    int64_t idx = base + i;
    v[i] = idx < n ? in[idx] : 0;
    s += v[i];
  }
  int64_t tot;
  int64_t ex = block_exclusive_scan(s, sh, &tot) + sums[blockIdx.x];
  for (int i = 0; i < kScanItems; ++i) {
    int64_t idx = base + i;
    if (idx < n) out[idx] = ex;
    ex += v[i];
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) out[n] = sums[gridDim.x];
}

}  // namespace

extern "C" size_t smx_scan_workspace(int64_t n) {
  int64_t tiles = (n + kScanTile - 1) / kScanTile;
  if (tiles < 1) tiles = 1;
  return size_t(tiles + 1) * sizeof(int64_t);
}

extern "C" int smx_scan_i64(const int64_t* in, int64_t* out, int64_t n, void* ws, size_t ws_bytes, void* stream) {
  SMX_REQUIRE(n >= 0 && out != nullptr && ws != nullptr, "smx_scan_i64: bad arguments");
  SMX_REQUIRE(n == 0 || in != nullptr, "smx_scan_i64: null input");
  SMX_REQUIRE(ws_bytes >= smx_scan_workspace(n), "smx_scan_i64: workspace too small");
  cudaStream_t st = smx::as_stream(stream);
  int64_t tiles = (n + kScanTile - 1) / kScanTile;
  if (tiles < 1) tiles = 1;
  int64_t* sums = static_cast<int64_t*>(ws);
  if (n == 0) {
    cudaMemsetAsync(out, 0, sizeof(int64_t), st);
    SMX_LAUNCH_CHECK("smx_scan_i64 memset");
    return SMX_OK;
  }
  scan_tile_sums<<<(unsigned)tiles, kScanBlock, 0, st>>>(in, n, sums);
  scan_sums_serial<<<1, 1024, 0, st>>>(sums, tiles);
  scan_tiles<<<(unsigned)tiles, kScanBlock, 0, st>>>(in, out, n, sums);
  SMX_LAUNCH_CHECK("smx_scan_i64");
  return SMX_OK;
}

extern "C" const char* smx_last_error_string(void) { return smx::g_last_error.c_str(); }

extern "C" const char* smx_version(void) { return "smolyax_gb300 0.1 (sm_103a)"; }

extern "C" int smx_host_device_pointer(const void* host, void** dev) {
  SMX_REQUIRE(host != nullptr && dev != nullptr, "smx_host_device_pointer: null pointer");
  *dev = nullptr;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, host) != cudaSuccess || at.type != cudaMemoryTypeHost) {
    cudaGetLastError();
    return smx::set_error(SMX_ERR_ARG, "smx_host_device_pointer: not page-locked host memory");
  }
  if (cudaHostGetDevicePointer(dev, const_cast<void*>(host), 0) != cudaSuccess || *dev == nullptr) {
    cudaGetLastError();
    *dev = nullptr;
    return smx::set_error(SMX_ERR_UNSUPPORTED, "smx_host_device_pointer: host memory not mapped for the device");
  }
  return SMX_OK;
}
