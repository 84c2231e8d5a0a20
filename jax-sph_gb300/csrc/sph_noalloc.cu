// sph_nl_edges_noalloc: the neighbour-list build without any device
// allocation, for callers that cannot call cudaMalloc -- e.g. a host
// framework that owns the whole device memory pool and forbids side
// allocations, or code that must not allocate after its start-up phase. The
// caller passes positions and the output edge list; every piece of scratch
// (cell counts and starts, sort keys, sorted positions, scan carries) lives in
// one file-scope device array of fixed size, so the build works for at most
// SPH_NOALLOC_MAX_PARTICLES particles and SPH_NOALLOC_MAX_CELLS cells.
//
// The array is shared by every call on a device and keeps the previous call's
// contents: each call clears what must start at zero (cell counts, status
// word) and overwrites the rest before reading it. Calls whose work overlaps
// on the GPU (different streams, or different host threads) race on the
// array; the caller must order them. The first call on each device looks the
// array's device address up (cudaGetSymbolAddress, with that device
// current); make that first call before any stream capture. The address is
// kept for the life of the process, so the device must not be reset
// (cudaDeviceReset) between calls: the module, and with it the array, would
// be loaded again elsewhere.
//
// Cost on dense inputs: ranking a particle within its cell (k_na_place) and
// ordering a sender's receivers (the insertion sort of the edge emission) are
// quadratic in the occupancy of a cell and of a neighbourhood; inputs that
// put thousands of particles into one cell make a call slow.
#include <mutex>

#include "sph_internal.cuh"

using namespace sph;

namespace {

constexpr long long kMaxN = SPH_NOALLOC_MAX_PARTICLES;
constexpr long long kMaxC = SPH_NOALLOC_MAX_CELLS;
constexpr int kBlock = 256;
constexpr unsigned kFull = 0xffffffffu;

constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }
// byte offsets of the scratch regions
constexpr size_t kCase = 0;
constexpr size_t kStatus = align256(kCase + sizeof(CaseDev));
constexpr size_t kCount = align256(kStatus + sizeof(unsigned));
constexpr size_t kStart = align256(kCount + sizeof(int) * (kMaxC + 1));
constexpr size_t kKeyc = align256(kStart + sizeof(int) * (kMaxC + 1));
constexpr size_t kKeys = align256(kKeyc + sizeof(int) * kMaxN);
constexpr size_t kTkey = align256(kKeys + sizeof(int) * kMaxN);
constexpr size_t kTcell = align256(kTkey + sizeof(int) * kMaxN);
constexpr size_t kOrig = align256(kTcell + sizeof(int) * kMaxN);
constexpr size_t kCellid = align256(kOrig + sizeof(int) * kMaxN);
constexpr size_t kMeta = align256(kCellid + sizeof(int) * kMaxN);
constexpr size_t kRowcnt = align256(kMeta + sizeof(int) * kMaxN);
constexpr size_t kRowoff = align256(kRowcnt + sizeof(int) * (kMaxN + 1));
constexpr size_t kScan = align256(kRowoff + sizeof(long long) * (kMaxN + 1));
constexpr size_t kScanInts = 4096;  // > scan_tmp_ints(kMaxN + 1) = 648 (64-bit sums)
constexpr size_t kP4 = align256(kScan + sizeof(int) * kScanInts);
constexpr size_t kBytes = align256(kP4 + sizeof(float4) * kMaxN);

static __device__ __align__(256) unsigned char g_nl_scratch[kBytes];

std::mutex g_mu;
constexpr int kMaxDevices = 256;
unsigned char* g_addr[kMaxDevices] = {};

int fail(int code, const char* msg) {
  set_last_error(msg);
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  set_last_error(std::string(what) + ": " + cudaGetErrorString(e));
  return (int)SPH_ERR_CUDA;
}

// Device address of the scratch array on the current device (looked up once
// per device, with that device current).
int scratch_address(unsigned char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return fail((int)SPH_ERR_INVALID_ARG, "device ordinal");
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_nl_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress");
    g_addr[dev] = (unsigned char*)p;
  }
  *out = g_addr[dev];
  return 0;
}

__global__ void k_na_setcase(CaseDev c, CaseDev* dst) { *dst = c; }

// Cell of each particle (original order) and its slot within the cell.
template <int DIM>
__global__ void k_na_hash(long long n, const float* __restrict__ r, const CaseDev* c, int* count,
                          int* keyc, int* keys, unsigned* status) {
  long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  bool valid = k < n;
  int cell = 0;
  if (valid) {
    float4 p = make_float4(r[k * DIM], r[k * DIM + 1], DIM == 3 ? r[k * DIM + 2] : 0.f, 0.f);
    cell = cell_hash<DIM>(p, *c, status);
  }
  unsigned mask = __ballot_sync(kFull, valid);
  if (!valid) return;
  unsigned peers = __match_any_sync(mask, cell);
  int lane = threadIdx.x & 31;
  int leader = __ffs(peers) - 1;
  int rank = __popc(peers & ((1u << lane) - 1u));
  int base = 0;
  if (lane == leader) base = atomicAdd(&count[cell], __popc(peers));
  base = __shfl_sync(peers, base, leader);
  keyc[k] = cell;
  keys[k] = base + rank;
}

__global__ void k_na_scatter(long long n, const int* keyc, const int* keys, const int* start,
                             int* tkey, int* tcell) {
  long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (k >= n) return;
  int cell = keyc[k];
  int q = start[cell] + keys[k];
  tkey[q] = (int)k;
  tcell[q] = cell;
}

// Sorted position of every particle: cell order, original index inside a cell.
template <int DIM>
__global__ void k_na_place(long long n, const float* __restrict__ r, const int* start,
                           const int* tkey, const int* tcell, float4* P4, int* orig, int* cellid,
                           int* meta) {
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= n) return;
  int cell = tcell[q];
  int a = start[cell], e = start[cell + 1];
  int key = tkey[q];
  int rank = 0;
  for (int t = a; t < e; ++t) rank += (tkey[t] < key);
  int dest = a + rank;
  P4[dest] = make_float4(r[(long long)key * DIM], r[(long long)key * DIM + 1],
                         DIM == 3 ? r[(long long)key * DIM + 2] : 0.f, 0.f);
  orig[dest] = key;
  cellid[dest] = cell;
  meta[dest] = 0;
}

}  // namespace

extern "C" {

int sph_nl_edges_noalloc(int32_t dim, const double* box, double r_cutoff, int32_t mask_self,
                         const float* r, int64_t n, int32_t* idx, int64_t capacity,
                         int64_t* count_dev, uint32_t* status_dev, void* stream) try {
  if (dim != 2 && dim != 3) return fail((int)SPH_ERR_INVALID_ARG, "dimension must be 2 or 3");
  if (!box || !r || !idx || !count_dev) return fail((int)SPH_ERR_INVALID_ARG, "null argument");
  if (n < 1 || n > kMaxN)
    return fail((int)SPH_ERR_INVALID_ARG,
                "particle count outside 1..SPH_NOALLOC_MAX_PARTICLES (65536)");
  if (capacity < 0 || capacity > (1LL << 40))
    return fail((int)SPH_ERR_INVALID_ARG, "bad edge capacity");
  SphConfig cfg{};
  cfg.dim = dim;
  cfg.mask_self = mask_self ? 1 : 0;
  cfg.capacity_multiplier = 1.25;
  SphCase sc{};
  sc.n = n;
  for (int d = 0; d < 3; ++d) sc.box[d] = d < dim ? box[d] : 1.0;
  sc.r_cutoff = r_cutoff;
  sc.dx = sc.h = r_cutoff;
  sc.eos = SPH_EOS_TAIT;
  sc.p_ref = sc.rho_ref = sc.gamma = sc.u_ref = 1.0;
  sc.eta_limiter = -1.0;
  CaseDev c;
  std::string err;
  if (make_case(cfg, sc, 0, 0, c, err, false)) return fail((int)SPH_ERR_INVALID_ARG, err.c_str());
  if (c.ncell > kMaxC)
    return fail((int)SPH_ERR_INVALID_ARG, "cell count above SPH_NOALLOC_MAX_CELLS (65536)");
  unsigned char* base = nullptr;
  int rc = scratch_address(&base);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  CaseDev* dcase = (CaseDev*)(base + kCase);
  unsigned* status = (unsigned*)(base + kStatus);
  int* count = (int*)(base + kCount);
  int* start = (int*)(base + kStart);
  int* keyc = (int*)(base + kKeyc);
  int* keys = (int*)(base + kKeys);
  int* tkey = (int*)(base + kTkey);
  int* tcell = (int*)(base + kTcell);
  Buffers b{};
  b.P4 = (float4*)(base + kP4);
  b.ORIG = (int*)(base + kOrig);
  b.META = (int*)(base + kMeta);
  int* cellid = (int*)(base + kCellid);
  int* rowcnt = (int*)(base + kRowcnt);
  long long* rowoff = (long long*)(base + kRowoff);
  int* scan_tmp = (int*)(base + kScan);

  const int g = (int)((n + kBlock - 1) / kBlock);
  k_na_setcase<<<1, 1, 0, st>>>(c, dcase);
  cudaMemsetAsync(status, 0, sizeof(unsigned), st);
  cudaMemsetAsync(count, 0, sizeof(int) * (c.ncell + 1), st);
  if (dim == 3)
    k_na_hash<3><<<g, kBlock, 0, st>>>(n, r, dcase, count, keyc, keys, status);
  else
    k_na_hash<2><<<g, kBlock, 0, st>>>(n, r, dcase, count, keyc, keys, status);
  launch_scan(st, count, start, c.ncell, scan_tmp);
  k_na_scatter<<<g, kBlock, 0, st>>>(n, keyc, keys, start, tkey, tcell);
  if (dim == 3)
    k_na_place<3><<<g, kBlock, 0, st>>>(n, r, start, tkey, tcell, b.P4, b.ORIG, cellid, b.META);
  else
    k_na_place<2><<<g, kBlock, 0, st>>>(n, r, start, tkey, tcell, b.P4, b.ORIG, cellid, b.META);
  LaunchCtx L{};
  L.stream = st;
  L.dim = dim;
  L.mask_self = cfg.mask_self;
  L.N = n;
  L.n_cases = 1;
  L.cases = dcase;
  L.status = status;
  launch_edges(L, b, cellid, start, rowcnt, rowoff, scan_tmp, idx, capacity, (long long*)count_dev);
  if (status_dev)
    cudaMemcpyAsync(status_dev, status, sizeof(unsigned), cudaMemcpyDeviceToDevice, st);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "sph_nl_edges_noalloc launch");
  return 0;
} catch (...) {
  return host_error();
}

}  // extern "C"
