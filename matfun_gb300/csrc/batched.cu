// batched.cu -- many requests of uneven size and mixed family / kind / order / precision in one launch.
//
// The host cuts every request into tiles (gmf: 128 matrices; smf: 64 or 128, matfun_cuda_batched_tune_tiles) and
// writes a table (requests, their coefficient blocks, the prefix sum of their tile counts; the general family's
// requests first) into device memory.  Two persistent kernels (grid = SMs x CTAs per SM) then pull tiles from their
// global atomic cursors until all are taken: batched_gmf_kernel the general family's, at the 3 CTAs per SM of the
// standalone gmf kernel, and batched_kernel the others, launched as a programmatic dependent of the first so that it
// fills the SMs the first one leaves as it drains.  Each tile runs the same tile routine as the standalone kernel of
// its request (smf FP64 / mixed FP32 in either layout, gmf FP64 / mixed FP32), by the CTA's 128 threads; a launch's
// dynamic shared memory is that of its largest tile.  There is no waiting between CTAs: a CTA only increments its
// cursor and stops when it passes the tile count, so no wait can hang.
//
// Two ways to run it:
//   matfun_cuda_batched(requests, count, stream)          table in a per-device cached buffer, uploaded on `stream`
// gmf requests of log / pow at orders 1, 2 (exp at order 2) with at least BT_SORT_MIN matrices are evaluated in the
// batch order of the
// standalone launch (by spectral class): their permutations are computed on the stream before the persistent kernel,
// into an order region after the table (in the cached buffer, or in the plan's allocation).
//   matfun_cuda_batched_plan / _run / _free                 table uploaded once; _run only clears the cursor and
//                                                           launches, so it can be captured in a CUDA graph
// The CTAs per SM, the order in which requests are laid out (as given, or longest tile work first) and the smf tile
// size come from matfun_cuda_batched_tune / _tune_tiles (set by the autotuner of matfun_gb300/autotune.py); a plan
// keeps the layout and tile size in force when it was made.
#include <algorithm>
#include <climits>
#include <cstddef>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/matfun_cuda.h"
#include "batched_tiles.cuh"

namespace mf {
namespace {

// dispatch of a tile to its variant
#define MF_SMF_CALL(pfx, K, suf)                                                        \
  switch (R.order) {                                                                    \
    case 2: pfx##_##K##_2_##suf(base, cnt, R, coef, smem); break;                        \
    case 1: pfx##_##K##_1_##suf(base, cnt, R, coef, smem); break;                        \
    default: pfx##_##K##_0_##suf(base, cnt, R, coef, smem); break;                       \
  }
#define MF_SMF_KIND(pfx, suf)                                                           \
  switch (R.kind) {                                                                     \
    case 0: MF_SMF_CALL(pfx, 0, suf) break;                                              \
    case 1: MF_SMF_CALL(pfx, 1, suf) break;                                              \
    case 3: MF_SMF_CALL(pfx, 3, suf) break;                                              \
    default: MF_SMF_CALL(pfx, 2, suf) break;                                             \
  }
#define MF_GMF_CALL(pfx, K)                                                             \
  switch (R.order) {                                                                    \
    case 2: pfx##_##K##_2(base, cnt, R, coef, smem); break;                              \
    case 1: pfx##_##K##_1(base, cnt, R, coef, smem); break;                              \
    default: pfx##_##K##_0(base, cnt, R, coef, smem); break;                             \
  }
#define MF_GMF_KIND(pfx)                \
  switch (R.kind) {                     \
    case 0: MF_GMF_CALL(pfx, 0) break;  \
    case 1: MF_GMF_CALL(pfx, 1) break;  \
    default: MF_GMF_CALL(pfx, 2) break; \
  }

__device__ void run_gmf_tile(const DevReq &R, long long base, int cnt, const unsigned char *coef,
                             unsigned char *smem) {
  if (R.dtype == 0) { MF_GMF_KIND(bt_gmf) } else { MF_GMF_KIND(bt_gmf32) }
}

__device__ void run_tile(const DevReq &R, long long base, int cnt, const unsigned char *coef, unsigned char *smem) {
  if (R.tile == BT_TPB) {
    if (R.family == 1) {
      if (R.dtype == 0) { MF_SMF_KIND(bt_smf64, m) } else { MF_SMF_KIND(bt_smf32, m) }
    } else {
      if (R.dtype == 0) { MF_SMF_KIND(bt_smf64, v) } else { MF_SMF_KIND(bt_smf32, v) }
    }
  } else {
    if (R.family == 1) {
      if (R.dtype == 0) { MF_SMF_KIND(bt_smf64, m64) } else { MF_SMF_KIND(bt_smf32, m64) }
    } else {
      if (R.dtype == 0) { MF_SMF_KIND(bt_smf64, v64) } else { MF_SMF_KIND(bt_smf32, v64) }
    }
  }
}

// the persistent loop over the tiles tile_start[0] .. tile_start[nreq] - 1 of requests reqs[0 .. nreq - 1]
template <bool GMF_ONLY>
__device__ __forceinline__ void batched_loop(const DevReq *__restrict__ reqs, int nreq,
                                             const long long *__restrict__ tile_start,
                                             unsigned long long *__restrict__ cursor,
                                             const unsigned char *__restrict__ coefs, unsigned char *smem) {
  __shared__ long long s_tile;
  const long long first = tile_start[0], total = tile_start[nreq];
  for (;;) {
    if (threadIdx.x == 0) s_tile = first + (long long)atomicAdd(cursor, 1ull);
    __syncthreads();
    const long long t = s_tile;
    __syncthreads();
    if (t >= total) break;
    int lo = 0, hi = nreq;  // request of tile t: tile_start[lo] <= t < tile_start[lo + 1]
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (tile_start[mid] <= t) lo = mid;
      else hi = mid;
    }
    const DevReq R = reqs[lo];
    const long long base = (t - tile_start[lo]) * R.tile;
    const int cnt = (int)min((long long)R.tile, R.n - base);
    if (GMF_ONLY) run_gmf_tile(R, base, cnt, coefs + R.coef_off, smem);
    else run_tile(R, base, cnt, coefs + R.coef_off, smem);
    __syncthreads();  // the tile's shared memory is reused by the next tile
  }
}

// every family (the symmetric tile routines take up to 255 registers: 2 CTAs per SM)
__global__ void __launch_bounds__(BT_TPB) batched_kernel(const DevReq *__restrict__ reqs, int nreq,
                                                         const long long *__restrict__ tile_start,
                                                         unsigned long long *__restrict__ cursor,
                                                         const unsigned char *__restrict__ coefs) {
  extern __shared__ __align__(16) unsigned char smem[];
  batched_loop<false>(reqs, nreq, tile_start, cursor, coefs, smem);
}

// the general family's requests, at the 3 CTAs per SM of the standalone gmf kernel (its tile routines are compiled
// for 168 registers); the launch that follows it on the stream may start once every CTA has started (the requests
// of one table are independent)
__global__ void __launch_bounds__(BT_TPB, GMF_MIN_CTAS) batched_gmf_kernel(const DevReq *__restrict__ reqs, int nreq,
                                                                          const long long *__restrict__ tile_start,
                                                                          unsigned long long *__restrict__ cursor,
                                                                          const unsigned char *__restrict__ coefs) {
  extern __shared__ __align__(16) unsigned char smem[];
  griddep_launch_dependents();
  batched_loop<true>(reqs, nreq, tile_start, cursor, coefs, smem);
}

// the dynamic shared memory of one request's tiles
size_t tile_smem(int family, int order, int dtype, int tile) {
  const bool mat = family == 1;
  if (family == 2) return sizeof(GmfSmem);
  if (tile == BT_TPB) {
    if (dtype == 0) return order == 2 ? (mat ? sizeof(SmfS<2, true>) : sizeof(SmfS<2, false>))
                                      : order == 1 ? (mat ? sizeof(SmfS<1, true>) : sizeof(SmfS<1, false>))
                                                   : (mat ? sizeof(SmfS<0, true>) : sizeof(SmfS<0, false>));
    return order == 2 ? (mat ? sizeof(SmfxS<2, true>) : sizeof(SmfxS<2, false>))
                      : order == 1 ? (mat ? sizeof(SmfxS<1, true>) : sizeof(SmfxS<1, false>))
                                   : (mat ? sizeof(SmfxS<0, true>) : sizeof(SmfxS<0, false>));
  }
  if (dtype == 0) return order == 2 ? (mat ? sizeof(SmfS<2, true, 64>) : sizeof(SmfS<2, false, 64>))
                                    : order == 1 ? (mat ? sizeof(SmfS<1, true, 64>) : sizeof(SmfS<1, false, 64>))
                                                 : (mat ? sizeof(SmfS<0, true, 64>) : sizeof(SmfS<0, false, 64>));
  return order == 2 ? (mat ? sizeof(SmfxS<2, true, 64>) : sizeof(SmfxS<2, false, 64>))
                    : order == 1 ? (mat ? sizeof(SmfxS<1, true, 64>) : sizeof(SmfxS<1, false, 64>))
                                 : (mat ? sizeof(SmfxS<0, true, 64>) : sizeof(SmfxS<0, false, 64>));
}

// the largest dynamic shared memory of any tile (the kernel's attribute is raised to it once per device)
constexpr size_t smem_max() {
  size_t m = sizeof(GmfSmem);
  m = std::max(m, sizeof(SmfS<2, true>));
  m = std::max(m, sizeof(SmfS<2, false>));
  m = std::max(m, sizeof(SmfxS<2, true>));
  return m;
}

// ------------------------------------------------------------------------------------------------ host side
struct Tuning {
  int ctas_per_sm = 2;
  int longest_first = 1;
  int smf_tile = BT_TPB;  // matrices per smf tile: 64 or 128
};
Tuning g_tune;

// a gmf request whose matrices are evaluated in the batch order of the standalone launch (log, pow at orders 1, 2;
// exp at order 2; at least BT_SORT_MIN matrices): its permutation, block histograms, their totals and keys lie at `off` of the order
// region that follows the table and the cursor
struct Ord {
  int req, kind, dtype;
  long long n;
  const void *x;
  size_t off;
};
constexpr long long BT_SORT_MIN = 2048;

struct Table {                  // a validated request list laid out for the device
  std::vector<unsigned char> bytes;  // DevReq[count] | tile_start[count + 1] | coefficient blocks
  size_t off_tiles = 0, off_coef = 0;
  int count = 0;
  std::vector<Ord> ords;
  size_t ord_bytes = 0;
  int gmf_count = 0;  // requests 0 .. gmf_count - 1 are the general family's (batched_gmf_kernel), the rest the others
  size_t smem = 0;    // dynamic shared memory of the launch of the other families: the largest of their tiles
};

size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }
long long key_blocks(long long n) { return (n + GKEY_TPB - 1) / GKEY_TPB; }
// order (4 n) | counts (4 GKEY_BINS blocks) | totals (4 GKEY_BINS) | keys (n bytes)
size_t ord_size(long long n) {
  return align16(4 * (size_t)n) + 4 * (size_t)GKEY_BINS * key_blocks(n) + 4 * (size_t)GKEY_BINS + align16((size_t)n);
}

// -1: invalid request (the rules of the single entry points), 0: ok
int build_table(const mf_request *req, int count, Table &T) {
  if (count < 0 || (count > 0 && !req)) return -1;
  struct Item {
    DevReq d;
    std::vector<unsigned char> coef;
    long long tiles;
    double work;
  };
  std::vector<Item> items;
  items.reserve(count);
  for (int i = 0; i < count; i++) {
    const mf_request &r = req[i];
    int kind = r.kind;
    double al = r.alpha;
    if (r.family < 0 || r.family > 2 || kind < SMF_EXP || kind > SMF_SQRT || r.order < 0 || r.order > 2 ||
        r.n < 0 || (r.dtype != 0 && r.dtype != 1) ||
        (kind == SMF_POW && !(al > 0)))
      return -1;
    if (r.n > 0 && (!r.x || !r.F || (r.order >= 1 && !r.J) || (r.order >= 2 && !r.H))) return -1;
    if (r.n > (long long)INT_MAX * 32) return -1;
    if (r.n == 0) continue;
    if (r.family == 2 && kind == SMF_SQRT) kind = SMF_POW, al = 0.5;
    if (kind != SMF_POW) al = kind == SMF_SQRT ? 0.5 : 0.0;
    Item it;
    it.d = DevReq{r.family, kind, r.order, r.dtype, al, (long long)r.n, r.x, r.F, r.order >= 1 ? r.J : nullptr,
                  r.order >= 2 ? r.H : nullptr, 0, nullptr, r.family == 2 ? BT_TPB : g_tune.smf_tile};
    if (r.family == 2) {
      GmfCoef C;
      gmf_coef(kind, al, r.order, C, r.dtype != 0);
      it.coef.resize(sizeof C);
      std::memcpy(it.coef.data(), &C, sizeof C);
    } else if (r.dtype == 0) {
      SmfCoef C;
      smf_coef(kind, al, C);
      it.coef.resize(sizeof C);
      std::memcpy(it.coef.data(), &C, sizeof C);
    } else {
      SmfCoefF C;
      smf_coef_f(kind, al, C);
      it.coef.resize(sizeof C);
      std::memcpy(it.coef.data(), &C, sizeof C);
    }
    it.tiles = (r.n + it.d.tile - 1) / it.d.tile;
    if (r.family != 2) T.smem = std::max(T.smem, tile_smem(r.family, r.order, r.dtype, it.d.tile));
    // relative work per matrix (measured orders of magnitude): gmf order 2 >> smf order 2 >> first orders
    const double per = (r.family == 2 ? 4.0 : 1.0) * (r.order == 2 ? 4.0 : (r.order == 1 ? 1.5 : 1.0)) *
                       (r.dtype == 1 ? (r.family == 2 ? 0.8 : 0.3) : 1.0);
    it.work = per * (double)r.n;
    items.push_back(std::move(it));
  }
  if (g_tune.longest_first)
    std::stable_sort(items.begin(), items.end(), [](const Item &a, const Item &b) { return a.work > b.work; });
  // the general family's requests first: their own persistent launch precedes that of the others
  std::stable_partition(items.begin(), items.end(), [](const Item &a) { return a.d.family == 2; });
  T.gmf_count = (int)std::count_if(items.begin(), items.end(), [](const Item &a) { return a.d.family == 2; });
  T.count = (int)items.size();
  T.off_tiles = align16(sizeof(DevReq) * T.count);
  T.off_coef = align16(T.off_tiles + sizeof(long long) * (T.count + 1));
  size_t coef_bytes = 0;
  for (auto &it : items) coef_bytes += align16(it.coef.size());
  T.bytes.assign(T.off_coef + coef_bytes, 0);
  long long tiles = 0;
  size_t co = 0;
  for (int i = 0; i < T.count; i++) {
    items[i].d.coef_off = (long long)co;
    std::memcpy(T.bytes.data() + sizeof(DevReq) * i, &items[i].d, sizeof(DevReq));
    std::memcpy(T.bytes.data() + T.off_tiles + sizeof(long long) * i, &tiles, sizeof tiles);
    std::memcpy(T.bytes.data() + T.off_coef + co, items[i].coef.data(), items[i].coef.size());
    tiles += items[i].tiles;
    co += align16(items[i].coef.size());
  }
  std::memcpy(T.bytes.data() + T.off_tiles + sizeof(long long) * T.count, &tiles, sizeof tiles);
  for (int i = 0; i < T.count; i++) {
    const DevReq &d = items[i].d;
    const bool kind_ok = (d.kind != SMF_EXP) | (d.order == 2);  // as the single gmf launch
    if ((d.family == 2) & kind_ok & (d.order >= 1) & (d.n >= BT_SORT_MIN) & (d.n <= INT_MAX)) {
      T.ords.push_back(Ord{i, d.kind, d.dtype, d.n, d.x, T.ord_bytes});
      T.ord_bytes += ord_size(d.n);
    }
  }
  return 0;
}

// the device address of each ordered request's permutation, written into its DevReq before the table is uploaded
void patch_idx(Table &T, unsigned char *ord_base) {
  for (const Ord &o : T.ords) {
    const int *idx = reinterpret_cast<const int *>(ord_base + o.off);
    std::memcpy(T.bytes.data() + sizeof(DevReq) * o.req + offsetof(DevReq, idx), &idx, sizeof idx);
  }
}

template <int KIND, typename T>
void launch_order(const Ord &o, unsigned char *ord_base, cudaStream_t st) {
  const int n = (int)o.n, nblk = (int)key_blocks(o.n);
  int *order = reinterpret_cast<int *>(ord_base + o.off);
  int *counts = reinterpret_cast<int *>(ord_base + o.off + align16(4 * (size_t)n));
  int *totals = counts + (size_t)GKEY_BINS * nblk;
  unsigned char *keys = reinterpret_cast<unsigned char *>(totals + GKEY_BINS);
  gmf_key_kernel<KIND, T><<<nblk, GKEY_TPB, 0, st>>>(n, static_cast<const T *>(o.x), keys, counts, nblk, nullptr);
  gmf_scan_kernel<<<GKEY_BINS, 1024, 0, st>>>(counts, nblk, totals);
  gmf_scatter_kernel<<<nblk, GKEY_TPB, 0, st>>>(n, keys, counts, totals, nblk, order);
}

// the permutations of the ordered requests (key, scan and scatter kernels of gmf_kernels.cuh), queued on `st` before
// the persistent kernel that reads them
cudaError_t launch_orders(const Table &T, unsigned char *ord_base, cudaStream_t st) {
  for (const Ord &o : T.ords) {
    if (o.dtype == 0) {
      if (o.kind == SMF_EXP) launch_order<EXP, double>(o, ord_base, st);
      else if (o.kind == SMF_LOG) launch_order<LOG, double>(o, ord_base, st);
      else launch_order<POW, double>(o, ord_base, st);
    } else {
      if (o.kind == SMF_EXP) launch_order<EXP, float>(o, ord_base, st);
      else if (o.kind == SMF_LOG) launch_order<LOG, float>(o, ord_base, st);
      else launch_order<POW, float>(o, ord_base, st);
    }
  }
  return cudaGetLastError();
}

cudaError_t prepare_kernel() {
  static std::atomic<unsigned long long> done{0}, done_g{0};  // one bit per device
  const cudaError_t e = smem_limit_per_device(batched_kernel, (int)smem_max(), done);
  return e != cudaSuccess ? e : smem_limit_per_device(batched_gmf_kernel, (int)sizeof(GmfSmem), done_g);
}

// cursors: two 8-byte counters (general family, the others) at `cursor`
cudaError_t launch_table(const unsigned char *dev_table, const Table &T, unsigned long long *cursor,
                         cudaStream_t st) {
  if (T.count == 0) return cudaSuccess;
  cudaError_t e = prepare_kernel();
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  e = cudaMemsetAsync(cursor, 0, 2 * sizeof(unsigned long long), st);
  if (e != cudaSuccess) return e;
  const DevReq *reqs = (const DevReq *)dev_table;
  const long long *tiles = (const long long *)(dev_table + T.off_tiles);
  const unsigned char *coefs = dev_table + T.off_coef;
  if (T.gmf_count > 0)
    batched_gmf_kernel<<<(unsigned)(sms * GMF_MIN_CTAS), BT_TPB, sizeof(GmfSmem), st>>>(reqs, T.gmf_count, tiles,
                                                                                       cursor, coefs);
  if (T.count > T.gmf_count) {
    // the other families' launch may start while the general family's drains (programmatic dependent launch)
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(sms * std::max(1, g_tune.ctas_per_sm)));
    cfg.blockDim = dim3(BT_TPB);
    cfg.dynamicSmemBytes = T.smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = T.gmf_count > 0 ? 1 : 0;
    e = cudaLaunchKernelEx(&cfg, batched_kernel, reqs + T.gmf_count, T.count - T.gmf_count, tiles + T.gmf_count,
                           cursor + 1, coefs);
    if (e != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

// true while `st` is being captured into a CUDA graph: the two batched entry points that take a request array
// upload it from a host copy that lives only until they return (and matfun_cuda_batched may reallocate its buffer),
// so they refuse a capturing stream; matfun_cuda_batched_plan / _run are the form to capture
bool capturing(cudaStream_t st) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  return cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone;
}

struct Plan {
  unsigned char *dev = nullptr;  // table, then the cursor
  Table table;
  size_t cursor_off = 0;
};

struct Scratch {  // per-device table buffer of matfun_cuda_batched
  std::mutex mu;
  unsigned char *dev = nullptr;
  size_t size = 0;
  cudaEvent_t last = nullptr;  // completion of the previous launch that used the buffer
};
Scratch g_scratch[64];

}  // namespace
}  // namespace mf

using namespace mf;

extern "C" int matfun_cuda_batched(const mf_request *requests, int count, void *stream) {
  Table T;
  if (build_table(requests, count, T) != 0) return -1;
  if (T.count == 0) return 0;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return -2;
  const cudaStream_t st = (cudaStream_t)stream;
  if (capturing(st)) return -1;
  Scratch &S = g_scratch[dev];
  std::lock_guard<std::mutex> lock(S.mu);
  const size_t ord_at = align16(T.bytes.size()) + 16;  // order region after the table and the cursor
  const size_t need = ord_at + T.ord_bytes;
  if (S.size < need) {
    if (S.dev) {
      if (S.last) cudaEventSynchronize(S.last);
      cudaFree(S.dev);
    }
    S.dev = nullptr;
    S.size = 0;
    if (cudaMalloc(&S.dev, need) != cudaSuccess) return -2;
    S.size = need;
  }
  if (!S.last && cudaEventCreateWithFlags(&S.last, cudaEventDisableTiming) != cudaSuccess) return -2;
  // the previous launch on another stream may still read the buffer: order this upload after it
  if (cudaStreamWaitEvent(st, S.last, 0) != cudaSuccess) return -2;
  patch_idx(T, S.dev + ord_at);
  // (a copy from pageable memory is staged before the call returns, so the host table may go out of scope)
  cudaError_t e = cudaMemcpyAsync(S.dev, T.bytes.data(), T.bytes.size(), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = launch_orders(T, S.dev + ord_at, st);
  if (e == cudaSuccess)
    e = launch_table(S.dev, T, (unsigned long long *)(S.dev + align16(T.bytes.size())), st);
  if (e == cudaSuccess) e = cudaEventRecord(S.last, st);
  return e == cudaSuccess ? 0 : -2;
}

extern "C" int matfun_cuda_batched_plan(const mf_request *requests, int count, void **plan) {
  if (!plan) return -1;
  *plan = nullptr;
  Plan *P = new Plan;
  if (build_table(requests, count, P->table) != 0) {
    delete P;
    return -1;
  }
  P->cursor_off = align16(P->table.bytes.size());
  const size_t ord_at = P->cursor_off + 16;
  const bool ok = cudaMalloc(&P->dev, ord_at + P->table.ord_bytes) == cudaSuccess;
  if (ok) patch_idx(P->table, P->dev + ord_at);
  if (!ok ||
      cudaMemcpy(P->dev, P->table.bytes.data(), P->table.bytes.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
    if (P->dev) cudaFree(P->dev);
    delete P;
    return -2;
  }
  *plan = P;
  return 0;
}

extern "C" int matfun_cuda_batched_run(void *plan, void *stream) {
  Plan *P = (Plan *)plan;
  if (!P) return -1;
  cudaError_t e = launch_orders(P->table, P->dev + P->cursor_off + 16, (cudaStream_t)stream);
  if (e == cudaSuccess)
    e = launch_table(P->dev, P->table, (unsigned long long *)(P->dev + P->cursor_off), (cudaStream_t)stream);
  return e == cudaSuccess ? 0 : -2;
}

extern "C" int matfun_cuda_batched_free(void *plan) {
  Plan *P = (Plan *)plan;
  if (!P) return 0;
  const cudaError_t e = P->dev ? cudaFree(P->dev) : cudaSuccess;
  delete P;
  return e == cudaSuccess ? 0 : -2;
}

extern "C" int matfun_cuda_batched_tune(int ctas_per_sm, int longest_first) {
  if (ctas_per_sm < 1 || ctas_per_sm > 8 || (longest_first != 0 && longest_first != 1)) return -1;
  g_tune.ctas_per_sm = ctas_per_sm;
  g_tune.longest_first = longest_first;
  return 0;
}

extern "C" int matfun_cuda_batched_tune_tiles(int smf_tile) {
  if (smf_tile != 64 && smf_tile != BT_TPB) return -1;
  g_tune.smf_tile = smf_tile;
  return 0;
}

// ------------------------------------------------------------------------------------------------ no allocation
// matfun_cuda_batched_noalloc: the same batched launch for callers that must not allocate device memory -- code that
// runs inside a host framework which owns every device allocation (its own caching allocator or memory pool), or a
// plugin that is only handed device arrays.  matfun_cuda_batched caches a table buffer it allocates with cudaMalloc;
// this entry point instead writes the request table and the tile cursor into one fixed array of device memory that
// is part of the library image (NOALLOC_BYTES, loaded with the library on every GPU that uses it and held until the
// process exits).  It calls no cudaMalloc, cudaFree or other device-allocating routine.  Having no room for the
// permutations, it evaluates gmf requests in their given order.
namespace {
constexpr size_t NOALLOC_BYTES = 256 * 1024;  // cursor (16 bytes) + request table: ~100 gmf or ~700 smf requests
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

std::mutex g_noalloc_mu;
unsigned char *g_noalloc_addr[64] = {};  // device address of g_noalloc_scratch, per device (set up on first use)
}  // namespace

extern "C" int matfun_cuda_batched_noalloc(const mf_request *requests, int count, void *stream) {
  Table T;
  if (build_table(requests, count, T) != 0) return -1;
  if (T.count == 0) return 0;
  if (16 + T.bytes.size() > NOALLOC_BYTES) return -4;  // the table does not fit the fixed scratch array
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return -2;
  const cudaStream_t st = (cudaStream_t)stream;
  if (capturing(st)) return -1;
  // The lock covers the set-up and the queueing of the table copy and the launch, so that two host threads calling
  // on the same stream queue copy A, launch A, copy B, launch B and never copy B before launch A.
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {  // first call on this device: the device address of the array, with it current
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return -2;
    g_noalloc_addr[dev] = (unsigned char *)p;
  }
  unsigned char *base = g_noalloc_addr[dev];
  // the cursor (first 16 bytes) is cleared by launch_table; the table follows it
  cudaError_t e = cudaMemcpyAsync(base + 16, T.bytes.data(), T.bytes.size(), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = launch_table(base + 16, T, (unsigned long long *)base, st);
  return e == cudaSuccess ? 0 : -2;
}
