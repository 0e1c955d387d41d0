// Allocation-free form of the tree field functor (tbslas_eval_tree_noalloc).
//
// Some callers cannot allocate device memory when they evaluate: code that
// runs under a fixed memory budget decided up front (a real-time or embedded
// solver loop), and code whose host application owns every device allocation
// through its own pool and forbids library-side cudaMalloc/cudaFree (both can
// synchronise the device and fragment the pool).  For them this entry point
// keeps its scratch (per-point leaf ids, per-leaf counts and offsets, the
// permutation and the tile list) in one file-scope device array of fixed
// size, TBSLAS_NOALLOC_SCRATCH_BYTES, which the CUDA module reserves on every
// GPU that loads this library until the process exits.  The entry point
// itself calls no cudaMalloc, cudaFree or allocating library routine.
#include <cuda.h>  // CUcontext/CUresult types; the two driver calls come through the runtime

#include <mutex>

#include "internal.h"
#include "tbslas_gb300.h"

namespace {

constexpr int64_t kMaxPoints = TBSLAS_NOALLOC_MAX_POINTS;
constexpr int64_t kMaxLeaves = TBSLAS_NOALLOC_MAX_LEAVES;
constexpr size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// Carve-up of the static array (each part 256-byte aligned).
constexpr size_t kOffLeafOf = 0;
constexpr size_t kOffCount = kOffLeafOf + align256(kMaxPoints * sizeof(int32_t));
constexpr size_t kOffCursor = kOffCount + align256(kMaxLeaves * sizeof(unsigned long long));
constexpr size_t kOffStart = kOffCursor + align256(kMaxLeaves * sizeof(unsigned long long));
constexpr size_t kOffNTile = kOffStart + align256((kMaxLeaves + 1) * sizeof(int64_t));
constexpr size_t kOffTileOff = kOffNTile + align256(kMaxLeaves * sizeof(int64_t));
constexpr size_t kOffPerm = kOffTileOff + align256((kMaxLeaves + 1) * sizeof(int64_t));
constexpr size_t kOffTiles = kOffPerm + align256(kMaxPoints * sizeof(int64_t));
constexpr size_t kTotal =
    kOffTiles + align256((kMaxPoints / tbg::kTile + 1 + kMaxLeaves) * sizeof(tbg::Tile));
static_assert(kTotal <= TBSLAS_NOALLOC_SCRATCH_BYTES, "scratch carve-up exceeds the stated size");

// The scratch.  Host code must not use this name as an address: on the host
// it is only a stand-in symbol; its device address comes from
// cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[TBSLAS_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
struct ScratchAddress {
  void* ptr = nullptr;
  unsigned long long context_id = 0;  // context the address was looked up in
};
ScratchAddress g_scratch_dev[kMaxDevices];

// Process-unique id of the calling thread's current context (0 when the
// driver cannot tell).  The driver never reuses an id, so a primary context
// that the host application destroyed (cudaDeviceReset) and the runtime
// created anew reads as a different context, and the array's address is
// looked up again in it.  The two driver functions are reached through the
// runtime's entry-point table; the library does not link the driver library.
unsigned long long current_context_id() {
  typedef CUresult (*GetCurrentFn)(CUcontext*);
  typedef CUresult (*GetIdFn)(CUcontext, unsigned long long*);
  static GetCurrentFn get_current = nullptr;
  static GetIdFn get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {  // under g_setup_mutex
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrentFn>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetIdFn>(f);
    cudaGetLastError();
    looked_up = true;
  }
  CUcontext c = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&c) != CUDA_SUCCESS || !c ||
      get_id(c, &id) != CUDA_SUCCESS)
    return 0;
  return id;
}

// Set-up, once per device and context, with that device current: the device
// address of the array (host code only knows a stand-in symbol for it).
int scratch_address(int device, unsigned char** out) {
  if (device < 0 || device >= kMaxDevices)
    return tbg::fail_status(TBSLAS_ERR_UNSUPPORTED, "device index outside the supported range");
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  const unsigned long long id = current_context_id();
  ScratchAddress& a = g_scratch_dev[device];
  if (!a.ptr || a.context_id != id) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      a.ptr = nullptr;
      return tbg::fail_status(TBSLAS_ERR_CUDA,
                              "cudaGetSymbolAddress of the no-alloc scratch array failed");
    }
    a.ptr = p;
    a.context_id = id;
  }
  *out = static_cast<unsigned char*>(a.ptr);
  return TBSLAS_OK;
}

}  // namespace

extern "C" int tbslas_eval_tree_noalloc(tbslas_tree tree, const double* pos_dev, int64_t n,
                                        double* out_dev, int bc, void* stream) {
  int64_t L = 0;
  int device = 0, dof = 0;
  int st = tbg::tree_shape(tree, &L, &device, &dof);
  if (st != TBSLAS_OK) return st;
  if (n < 0) return tbg::fail_status(TBSLAS_ERR_INVALID_ARG, "negative point count");
  if (n > kMaxPoints)
    return tbg::fail_status(TBSLAS_ERR_SIZE,
                            "tbslas_eval_tree_noalloc: more than TBSLAS_NOALLOC_MAX_POINTS "
                            "points; split the call or use tbslas_eval_tree");
  if (L > kMaxLeaves)
    return tbg::fail_status(TBSLAS_ERR_SIZE,
                            "tbslas_eval_tree_noalloc: tree has more than "
                            "TBSLAS_NOALLOC_MAX_LEAVES leaves; use tbslas_eval_tree");
  if (n > 0 && (!pos_dev || !out_dev))
    return tbg::fail_status(TBSLAS_ERR_INVALID_ARG, "null buffer");
  if (bc != TBSLAS_BC_FREESPACE && bc != TBSLAS_BC_PERIODIC)
    return tbg::fail_status(TBSLAS_ERR_INVALID_ARG, "invalid boundary condition");
  tbg::DeviceRestore restore;
  if (cudaSetDevice(device) != cudaSuccess)
    return tbg::fail_status(TBSLAS_ERR_CUDA, "cudaSetDevice failed");
  unsigned char* base = nullptr;
  st = scratch_address(device, &base);
  if (st != TBSLAS_OK) return st;
  tbg::BucketScratch b;
  b.leaf_of = reinterpret_cast<int32_t*>(base + kOffLeafOf);
  b.count = reinterpret_cast<unsigned long long*>(base + kOffCount);
  b.cursor = reinterpret_cast<unsigned long long*>(base + kOffCursor);
  b.start = reinterpret_cast<int64_t*>(base + kOffStart);
  b.ntile = reinterpret_cast<int64_t*>(base + kOffNTile);
  b.tileoff = reinterpret_cast<int64_t*>(base + kOffTileOff);
  b.perm = reinterpret_cast<int64_t*>(base + kOffPerm);
  b.tiles = reinterpret_cast<tbg::Tile*>(base + kOffTiles);
  return tbg::bucketed_eval_on(b, tree, pos_dev, n, out_dev, bc, (cudaStream_t)stream);
}
