// Neighbour-search integer stages: device exclusive scan, stable LSD radix sort of
// (cell, particle id) pairs, and the cell-start table.
//
// The reference executes an equation as `for i in 0..n { for j in 0..n { body } }`
// (prestige/src/codegen/simple_cpu.rs:7-8).  These stages replace the inner all-pairs loop
// by a cell list: particles are ordered by (cell, id) and cell c owns the slots
// cell_start[c] .. cell_start[c+1].  Everything here is integer work and bit-exact against
// the oracle's stable counting sort.
//
// Sort: 8-bit digits, least significant first.  Each pass is three launches:
//   digit_hist   per tile of 1024 keys (4096 without allocation), a 256-bin histogram
//                                                                   -> hist[d * tiles + t]
//   digit_scan   per digit, exclusive scan over tiles (in place)    -> digit_total[d]
//   digit_scatter stable per-tile ranking with warp match masks, then scatter
// Input order is id order, and every pass is stable, so equal cells stay in id order.
#include <cuda_runtime.h>

#include <mutex>

#include "pg_internal.cuh"

namespace pg {

namespace {

constexpr int kSortThreads = 256;
// Keys per thread of the histogram and scatter kernels.  The handles' sorts use 4 (tiles of 1024
// keys): against 16 (tiles of 4096) the 200,000-sphere DEM step went from 0.144 to 0.122 ms
// (49 tiles had left most of the 152 SMs idle) and the 4M-particle neighbour search from 0.304
// to 0.285 ms.  The no-allocation path keeps 16: its fixed scratch holds the histograms of
// 4096-key tiles.  The sort result does not depend on the tile size.  Digits of 10 bits, which
// sort the 19-bit DEM keys in two passes instead of three, were measured and dropped: the
// 1024-bin tables made each pass dearer by as much (DEM step 0.099 against 0.097 ms).
constexpr int kSortItems = 16;
constexpr int kSortItemsSmall = 4;
constexpr size_t kSmallSortN = ~size_t(0);
constexpr int kSortTile = kSortThreads * kSortItems;  // 4096 keys per tile
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kRadix = 256;

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;  // 4096 values per block

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// Block-wide exclusive scan of one value per thread (blockDim.x multiple of 32, <= 1024).
// Returns the exclusive prefix; *total receives the block sum.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* total) {
  __shared__ uint32_t warp_sums[32];
  __shared__ uint32_t block_total;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  uint32_t incl = warp_incl_scan(v);
  if (lane == 31) warp_sums[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t s = lane < nwarps ? warp_sums[lane] : 0u;
    uint32_t si = warp_incl_scan(s);
    if (lane < nwarps) warp_sums[lane] = si - s;
    if (lane == nwarps - 1) block_total = si;
  }
  __syncthreads();
  uint32_t r = incl - v + warp_sums[warp];
  if (total) *total = block_total;
  __syncthreads();
  return r;
}

// ---------------------------------------------------------------------------------------
// Exclusive scan (reduce, scan block sums, rescan).  out[m] receives the total.
// ---------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kScanThreads) scan_reduce_kernel(const uint32_t* __restrict__ in, size_t m,
                                                                   uint32_t* __restrict__ bsum) {
  const size_t base = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanItems;
  uint32_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k)
    if (base + k < m) s += in[base + k];
  uint32_t total;
  block_excl_scan(s, &total);
  if (threadIdx.x == 0) bsum[blockIdx.x] = total;
}

// One block scans the block sums sequentially in chunks of kScanThreads (any count).
__global__ void __launch_bounds__(kScanThreads) scan_bsum_kernel(uint32_t* __restrict__ bsum, size_t nb) {
  uint32_t carry = 0;
  for (size_t c0 = 0; c0 < nb; c0 += kScanThreads) {
    const size_t i = c0 + threadIdx.x;
    uint32_t v = i < nb ? bsum[i] : 0u;
    uint32_t total;
    uint32_t ex = block_excl_scan(v, &total);
    if (i < nb) bsum[i] = ex + carry;
    carry += total;
  }
}

__global__ void __launch_bounds__(kScanThreads) scan_apply_kernel(const uint32_t* __restrict__ in, size_t m,
                                                                  const uint32_t* __restrict__ bsum,
                                                                  uint32_t* __restrict__ out) {
  const size_t base = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanItems;
  uint32_t v[kScanItems];
  uint32_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    v[k] = base + k < m ? in[base + k] : 0u;
    s += v[k];
  }
  uint32_t total;
  uint32_t ex = block_excl_scan(s, &total) + bsum[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    if (base + k < m) out[base + k] = ex;
    ex += v[k];
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) out[m] = bsum[blockIdx.x] + total;
}

// ---------------------------------------------------------------------------------------
// Radix sort passes.
// ---------------------------------------------------------------------------------------
template <int ITEMS>
__global__ void __launch_bounds__(kSortThreads) digit_hist_kernel(const uint32_t* __restrict__ keys, size_t n,
                                                                  int shift, int tiles,
                                                                  uint32_t* __restrict__ hist) {
  __shared__ uint32_t cnt[kRadix];
  cnt[threadIdx.x] = 0;
  __syncthreads();
  const size_t base = (size_t)blockIdx.x * (kSortThreads * ITEMS);
#pragma unroll 4
  for (int it = 0; it < ITEMS; ++it) {
    const size_t i = base + (size_t)it * kSortThreads + threadIdx.x;
    if (i < n) atomicAdd(&cnt[(keys[i] >> shift) & 0xffu], 1u);
  }
  __syncthreads();
  hist[(size_t)threadIdx.x * tiles + blockIdx.x] = cnt[threadIdx.x];
}

// Block d: exclusive scan of hist[d * tiles .. + tiles) in place; total -> digit_total[d].
__global__ void __launch_bounds__(kSortThreads) digit_scan_kernel(uint32_t* __restrict__ hist, int tiles,
                                                                  uint32_t* __restrict__ digit_total) {
  uint32_t* row = hist + (size_t)blockIdx.x * tiles;
  uint32_t carry = 0;
  for (int c0 = 0; c0 < tiles; c0 += kSortThreads) {
    const int i = c0 + threadIdx.x;
    uint32_t v = i < tiles ? row[i] : 0u;
    uint32_t total;
    uint32_t ex = block_excl_scan(v, &total);
    if (i < tiles) row[i] = ex + carry;
    carry += total;
  }
  if (threadIdx.x == 0) digit_total[blockIdx.x] = carry;
}

// Stable scatter of one tile of 256 * ITEMS keys.  Warp w owns the w-th run of 32 * ITEMS keys
// and walks it in ITEMS rounds of 32; within a round, lanes with equal digits are ranked by lane
// (match mask), and a per-warp running count per digit carries the rank across rounds.
// Warps are then ordered by an exclusive scan of the per-warp counts per digit.
template <int ITEMS>
__global__ void __launch_bounds__(kSortThreads) digit_scatter_kernel(
    const uint32_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in, uint32_t* __restrict__ keys_out,
    uint32_t* __restrict__ vals_out, size_t n, int shift, int tiles, const uint32_t* __restrict__ hist,
    const uint32_t* __restrict__ digit_total) {
  __shared__ uint32_t wcnt[kSortWarps][kRadix];
  __shared__ uint32_t tile_off[kRadix];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // global offset of digit d in this tile = (sum of smaller digits) + (this digit in earlier tiles)
  {
    uint32_t total;
    uint32_t dbase = block_excl_scan(digit_total[tid], &total);
    tile_off[tid] = dbase + hist[(size_t)tid * tiles + blockIdx.x];
  }
#pragma unroll
  for (int w = 0; w < kSortWarps; ++w) wcnt[w][tid] = 0;
  __syncthreads();

  const size_t base = (size_t)blockIdx.x * (kSortThreads * ITEMS) + (size_t)warp * (32 * ITEMS);
  const uint32_t lt_mask = (1u << lane) - 1u;
  uint32_t key[ITEMS], val[ITEMS], rank[ITEMS];
#pragma unroll
  for (int r = 0; r < ITEMS; ++r) {
    const size_t i = base + (size_t)r * 32 + lane;
    const bool valid = i < n;
    key[r] = valid ? keys_in[i] : 0u;
    val[r] = valid ? vals_in[i] : 0u;
    const uint32_t dkey = valid ? ((key[r] >> shift) & 0xffu) : 0x100u;
    const uint32_t peers = __match_any_sync(0xffffffffu, dkey);
    const int leader = __ffs(peers) - 1;
    uint32_t old = 0;
    if (valid && lane == leader) {
      old = wcnt[warp][dkey];
      wcnt[warp][dkey] = old + __popc(peers);
    }
    old = __shfl_sync(0xffffffffu, old, leader);
    rank[r] = old + __popc(peers & lt_mask);
    __syncwarp();
  }
  __syncthreads();
  {  // per digit: exclusive scan over warps
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) {
      const uint32_t t = wcnt[w][tid];
      wcnt[w][tid] = run;
      run += t;
    }
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < ITEMS; ++r) {
    const size_t i = base + (size_t)r * 32 + lane;
    if (i < n) {
      const uint32_t d = (key[r] >> shift) & 0xffu;
      const uint32_t pos = tile_off[d] + wcnt[warp][d] + rank[r];
      keys_out[pos] = key[r];
      vals_out[pos] = val[r];
    }
  }
}

// cell_start[c] = first sorted slot whose cell is >= c, for c = 0 .. ncells (so cell_start[ncells]
// = n), by a binary search over the sorted cells: one kernel, no count buffer and no scan.  The
// threads of a warp search for consecutive cells, so they load the same midpoints on most steps.
__global__ void cell_start_kernel(const uint32_t* __restrict__ cell, uint32_t n, uint32_t ncells,
                                  uint32_t* __restrict__ start) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c > ncells) return;
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    const uint32_t mid = lo + (hi - lo) / 2;
    if (__ldg(cell + mid) < c) lo = mid + 1;
    else hi = mid;
  }
  start[c] = lo;
}

int bits_needed(uint64_t v) {
  int b = 0;
  while (v) {
    ++b;
    v >>= 1;
  }
  return b;
}

}  // namespace

size_t scan_tmp_words(size_t m) { return (m + kScanTile - 1) / kScanTile + 1; }

int launch_exclusive_scan(cudaStream_t st, const uint32_t* in, uint32_t* out, size_t m, uint32_t* tmp) {
  if (m == 0) {
    PG_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(uint32_t), st));
    return PG_OK;
  }
  const size_t nb = (m + kScanTile - 1) / kScanTile;
  scan_reduce_kernel<<<(unsigned)nb, kScanThreads, 0, st>>>(in, m, tmp);
  scan_bsum_kernel<<<1, kScanThreads, 0, st>>>(tmp, nb);
  scan_apply_kernel<<<(unsigned)nb, kScanThreads, 0, st>>>(in, m, tmp, out);
  PG_CUDA_TRY(cudaGetLastError());
  return PG_OK;
}

int NbrWork::init(size_t n_, uint64_t ncells_) {
  n = n_;
  ncells = ncells_;
  const int bits = bits_needed(ncells ? ncells - 1 : 0);
  passes = (bits + 7) / 8;
  items = n <= kSmallSortN ? kSortItemsSmall : kSortItems;
  const size_t tile = (size_t)kSortThreads * items;
  tiles = (int)((n + tile - 1) / tile);
  if (tiles < 1) tiles = 1;
  const size_t nn = n ? n : 1;
  PG_TRY(keys[0].ensure(nn * 4));
  PG_TRY(keys[1].ensure(nn * 4));
  PG_TRY(vals[0].ensure(nn * 4));
  PG_TRY(vals[1].ensure(nn * 4));
  PG_TRY(hist.ensure((size_t)kRadix * tiles * 4));
  PG_TRY(digit_total.ensure(kRadix * 4));
  PG_TRY(cell_start.ensure((ncells + 1) * 4));
  return PG_OK;
}

size_t NbrWork::bytes() const {
  return keys[0].bytes + keys[1].bytes + vals[0].bytes + vals[1].bytes + hist.bytes + digit_total.bytes +
         cell_start.bytes;
}

int sort_and_table(cudaStream_t st, NbrWork& w) {
  const size_t n = w.n;
  int cur = 0;
  for (int p = 0; p < w.passes; ++p) {
    const int shift = 8 * p;
    if (w.items == kSortItemsSmall)
      digit_hist_kernel<kSortItemsSmall><<<w.tiles, kSortThreads, 0, st>>>(w.keys[cur].as<uint32_t>(), n, shift,
                                                                          w.tiles, w.hist.as<uint32_t>());
    else
      digit_hist_kernel<kSortItems><<<w.tiles, kSortThreads, 0, st>>>(w.keys[cur].as<uint32_t>(), n, shift, w.tiles,
                                                                     w.hist.as<uint32_t>());
    digit_scan_kernel<<<kRadix, kSortThreads, 0, st>>>(w.hist.as<uint32_t>(), w.tiles, w.digit_total.as<uint32_t>());
    if (w.items == kSortItemsSmall)
      digit_scatter_kernel<kSortItemsSmall><<<w.tiles, kSortThreads, 0, st>>>(
          w.keys[cur].as<uint32_t>(), w.vals[cur].as<uint32_t>(), w.keys[cur ^ 1].as<uint32_t>(),
          w.vals[cur ^ 1].as<uint32_t>(), n, shift, w.tiles, w.hist.as<uint32_t>(), w.digit_total.as<uint32_t>());
    else
      digit_scatter_kernel<kSortItems><<<w.tiles, kSortThreads, 0, st>>>(
          w.keys[cur].as<uint32_t>(), w.vals[cur].as<uint32_t>(), w.keys[cur ^ 1].as<uint32_t>(),
          w.vals[cur ^ 1].as<uint32_t>(), n, shift, w.tiles, w.hist.as<uint32_t>(), w.digit_total.as<uint32_t>());
    cur ^= 1;
  }
  w.sorted_cell = w.keys[cur].as<uint32_t>();
  w.sorted_id = w.vals[cur].as<uint32_t>();
  // cell table: start[c] = first slot of cell c (start[ncells] = n)
  cell_start_kernel<<<(unsigned)((w.ncells + 1 + 255) / 256), 256, 0, st>>>(w.sorted_cell, (uint32_t)n,
                                                                          (uint32_t)w.ncells,
                                                                          w.cell_start.as<uint32_t>());
  PG_CUDA_TRY(cudaGetLastError());
  return PG_OK;
}

// =========================================================================================
// Cell list without device allocation (pg_cell_list_noalloc).
//
// The radix sort above needs scratch beyond its inputs and outputs: a second key/value buffer
// for the ping-pong passes, the per-tile digit histograms and the digit totals.  Handles get
// that scratch from cudaMalloc when they are created.  This variant takes it from one
// file-scope device array instead, so a call allocates nothing.  Its size fixes the largest
// system it accepts (kNoAllocMaxParticles).
//
// The array is shared by every call on a device and keeps the previous call's contents.
// Nothing in it needs to start at zero: the hash writes every key, each histogram launch
// writes every bin of its tiles, the digit scan writes every total.  Calls whose work
// overlaps on the GPU (different streams, or different host threads without ordering) race
// on it.
// =========================================================================================
namespace {

constexpr size_t kNoAllocMaxParticles = 1u << 20;
constexpr size_t kNoAllocMaxTiles = (kNoAllocMaxParticles + kSortTile - 1) / kSortTile;
constexpr size_t kNoAllocKeysOff = 0;
constexpr size_t kNoAllocValsOff = kNoAllocKeysOff + 4 * kNoAllocMaxParticles;
constexpr size_t kNoAllocHistOff = kNoAllocValsOff + 4 * kNoAllocMaxParticles;
constexpr size_t kNoAllocTotalOff = kNoAllocHistOff + 4 * kRadix * kNoAllocMaxTiles;
constexpr size_t kNoAllocBytes = kNoAllocTotalOff + 4 * kRadix;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_addr[kNoAllocMaxDevices] = {};

// Device address of the scratch array on the current device.  The array's name in host code
// is only a host-side stand-in.  A call made outside stream capture looks the address up with
// the device current (so a cudaDeviceReset, or another context made current, is picked up) and
// keeps it per device; a call made while `st` is capturing uses the kept address of the last
// call outside capture on this device, since a lookup may have to load the module, which
// capture forbids.
int noalloc_scratch(cudaStream_t st, unsigned char** out) {
  int dev = 0;
  PG_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNoAllocMaxDevices) {
    set_error("device ordinal %d is beyond the %d devices the no-allocation cell list supports", dev,
              kNoAllocMaxDevices);
    return PG_EINVAL;
  }
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cap) != cudaSuccess) {
    cudaGetLastError();  // the query itself is refused while another stream captures
    cap = cudaStreamCaptureStatusActive;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (cap == cudaStreamCaptureStatusNone) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      set_error("cudaGetSymbolAddress of the cell-list scratch failed: %s", cudaGetErrorString(e));
      return PG_ECUDA;
    }
    g_noalloc_addr[dev] = p;
  } else if (!g_noalloc_addr[dev]) {
    set_error("the first no-allocation cell list call on device %d was made during stream capture; "
              "make one call on the device before capturing", dev);
    return PG_ESTATE;
  }
  *out = (unsigned char*)g_noalloc_addr[dev];
  return PG_OK;
}

// Cell index of every particle (f64 positions, id order), the same arithmetic as hash_kernel:
// c_d = clamp(floor((x_d - lo_d) * inv), 0, n_d - 1), one IEEE subtraction then one product.
struct NoAllocGrid {
  double lo[3];
  double inv;
  int n[3];
  int dim;
};

__global__ void noalloc_hash_kernel(NoAllocGrid g, const double* __restrict__ pos, uint32_t n,
                                    uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int c[3] = {0, 0, 0};
  for (int d = 0; d < g.dim; ++d) {
    const double t = __dmul_rn(__dsub_rn(pos[(size_t)i * g.dim + d], g.lo[d]), g.inv);
    c[d] = !(t >= 0.0) ? 0 : (t >= (double)g.n[d] ? g.n[d] - 1 : (int)t);
  }
  keys[i] = ((uint32_t)c[2] * (uint32_t)g.n[1] + (uint32_t)c[1]) * (uint32_t)g.n[0] + (uint32_t)c[0];
  vals[i] = i;
}

// start[c] = first slot whose cell is >= c (c = 0 .. ncells), by binary search over the
// sorted cells, so every entry is written without a count buffer.
__global__ void noalloc_cell_start_kernel(const uint32_t* __restrict__ cell, uint32_t n, uint32_t ncells,
                                          uint32_t* __restrict__ start) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c > ncells) return;
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    const uint32_t mid = lo + (hi - lo) / 2;
    if (cell[mid] < c) lo = mid + 1;
    else hi = mid;
  }
  start[c] = lo;
}

}  // namespace

}  // namespace pg

extern "C" int pg_cell_list_noalloc(const double* pos, size_t n, int dim, const double domain_lo[3],
                                    const double domain_hi[3], double support, double cell_multiplier,
                                    uint32_t* sorted_cell, uint32_t* sorted_id, uint32_t* cell_start,
                                    size_t cell_start_capacity, size_t* n_cells, void* stream) {
  using namespace pg;
  clear_error();
  if (dim != 2 && dim != 3) {
    set_error("dim must be 2 or 3 (got %d)", dim);
    return PG_EINVAL;
  }
  if (!domain_lo || !domain_hi) {
    set_error("null domain bounds");
    return PG_EINVAL;
  }
  if (n > kNoAllocMaxParticles) {
    set_error("%zu particles exceed the %zu-particle limit of the no-allocation cell list", n,
              kNoAllocMaxParticles);
    return PG_EINVAL;
  }
  Grid g;
  PG_TRY(make_grid(dim, domain_lo, domain_hi, support, cell_multiplier, &g));
  const uint64_t nc = g.ncells();
  if (n_cells) *n_cells = (size_t)nc;
  if (!cell_start || cell_start_capacity < nc + 1) {
    set_error("cell_start needs %llu entries (capacity %zu)", (unsigned long long)(nc + 1), cell_start_capacity);
    return PG_EINVAL;
  }
  if (n && (!pos || !sorted_cell || !sorted_id)) {
    set_error("null position or output buffer");
    return PG_EINVAL;
  }
  unsigned char* scratch = nullptr;
  PG_TRY(noalloc_scratch((cudaStream_t)stream, &scratch));
  cudaStream_t st = (cudaStream_t)stream;
  if (n) {
    uint32_t* tmp_keys = (uint32_t*)(scratch + kNoAllocKeysOff);
    uint32_t* tmp_vals = (uint32_t*)(scratch + kNoAllocValsOff);
    uint32_t* hist = (uint32_t*)(scratch + kNoAllocHistOff);
    uint32_t* digit_total = (uint32_t*)(scratch + kNoAllocTotalOff);
    const int passes = (bits_needed(nc ? nc - 1 : 0) + 7) / 8;
    const int tiles = (int)((n + kSortTile - 1) / kSortTile);
    // Ping-pong between the scratch pair and the caller's outputs, starting on the side that
    // makes the last pass land in the outputs.
    uint32_t* kbuf[2] = {tmp_keys, sorted_cell};
    uint32_t* vbuf[2] = {tmp_vals, sorted_id};
    int cur = (passes % 2 == 0) ? 1 : 0;
    NoAllocGrid ng;
    for (int d = 0; d < 3; ++d) {
      ng.lo[d] = g.lo[d];
      ng.n[d] = g.n[d];
    }
    ng.inv = 1.0 / g.cell;
    ng.dim = dim;
    noalloc_hash_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(ng, pos, (uint32_t)n, kbuf[cur], vbuf[cur]);
    for (int p = 0; p < passes; ++p) {
      const int shift = 8 * p;
      digit_hist_kernel<kSortItems><<<tiles, kSortThreads, 0, st>>>(kbuf[cur], n, shift, tiles, hist);
      digit_scan_kernel<<<kRadix, kSortThreads, 0, st>>>(hist, tiles, digit_total);
      digit_scatter_kernel<kSortItems><<<tiles, kSortThreads, 0, st>>>(kbuf[cur], vbuf[cur], kbuf[cur ^ 1],
                                                                       vbuf[cur ^ 1], n, shift, tiles, hist,
                                                                       digit_total);
      cur ^= 1;
    }
  }
  noalloc_cell_start_kernel<<<(unsigned)((nc + 1 + 255) / 256), 256, 0, st>>>(sorted_cell, (uint32_t)n, (uint32_t)nc,
                                                                             cell_start);
  PG_CUDA_TRY(cudaGetLastError());
  return PG_OK;
}
