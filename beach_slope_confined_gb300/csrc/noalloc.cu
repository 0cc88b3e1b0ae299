// noalloc.cu -- bsc_csr_solve_noalloc: the standalone BiCGSTAB solve of
// bsc_csr_solve for callers that may not allocate device memory.
//
// Who needs it: a host program that owns the GPU's memory budget -- a
// simulation that reserves HBM up front in its own pool, or a framework whose
// caching allocator holds most of the device -- cannot let a library call
// cudaMalloc/cudaFree inside its time loop: the call may fail for lack of
// memory the pool already holds, and cudaFree synchronises the whole device.
// Such a caller keeps the matrix and vectors in its own device memory and
// passes those pointers here.
//
// The Krylov work vectors, reduction partials, solver scalars and the
// last-block ticket live in one file-scope __device__ array of fixed size
// (rows <= BSC_NOALLOC_MAX_ROWS).  Host code only names the array; its device
// address on the current device comes from cudaGetSymbolAddress.  The lookup
// is repeated on every call (a host-side table lookup once the module is
// loaded), so an address never outlives the context it came from: after a
// cudaDeviceReset the module loads again, possibly elsewhere.  Under CUDA's
// lazy module loading the first call on a device loads this module, which is
// when the array's memory is committed.  Every call shares the array and
// leaves its contents behind, so the ticket and the scalars are cleared at
// the start of each call; two calls whose work overlaps on the GPU (two
// streams, or two host threads) race on the array, and on the one host-side
// copy of the solver scalars, which is process-wide.
#include "bsc_internal.cuh"

namespace bsc {
namespace {

constexpr size_t kVecBytes = (size_t)BSC_NOALLOC_MAX_ROWS * sizeof(double);
constexpr size_t round256(size_t b) { return (b + 255) & ~(size_t)255; }
// layout of the scratch array, every region on a 256-byte boundary
constexpr size_t kOffWork = 0;                                        // r rh p v s t (6 vectors)
constexpr size_t kOffPart = kOffWork + 6 * kVecBytes;                // partials, 8 x RED_GRID
constexpr size_t kOffHd = kOffPart + round256(8 * RED_GRID * sizeof(double));  // residual norms
constexpr size_t kOffSc = kOffHd + round256(64 * sizeof(double));    // device scalars
constexpr size_t kOffTicket = kOffSc + round256(sizeof(Scalars));    // last-block ticket
constexpr size_t kScratchBytes = kOffTicket + 256;

Scalars g_host_scalars;  // host copy read between iteration batches (process-wide)

}  // namespace

// the scratch itself: about 6.3 MB of device memory on every device that
// loads this module, held until the process exits
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// device address of g_scratch on the current device
static int scratch_address(unsigned char** out) {
    void* ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_scratch) != cudaSuccess || !ptr) {
        (void)cudaGetLastError();
        return BSC_E_CUDA;
    }
    *out = static_cast<unsigned char*>(ptr);
    return BSC_OK;
}

// true for memory the kernels on device `dev` may read and write directly:
// device memory of that device, or managed memory
static bool device_pointer(const void* p, int dev) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        (void)cudaGetLastError();
        return false;
    }
    if (a.type == cudaMemoryTypeManaged) return true;
    return a.type == cudaMemoryTypeDevice && a.device == dev;
}

}  // namespace bsc

using namespace bsc;

extern "C" {

int bsc_csr_solve_noalloc(const bsc_params* p, int32_t n, const int32_t* rowptr, const int32_t* col,
                          const double* val, const double* b, double* x, void* stream, bsc_solve_info* info) {
    if (!p || !rowptr || !col || !val || !b || !x || !info || n <= 0) return BSC_E_INVALID;
    if (n > BSC_NOALLOC_MAX_ROWS) return BSC_E_CAPACITY;
    if (p->solver != BSC_SOLVER_BICGSTAB) return BSC_E_INVALID;
    int ndev = 0, dev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        (void)cudaGetLastError();
        return BSC_E_NOT_BUILT;
    }
    if (cudaGetDevice(&dev) != cudaSuccess) {
        (void)cudaGetLastError();
        return BSC_E_CUDA;
    }
    const void* ptrs[] = {rowptr, col, val, b, x};
    for (const void* q : ptrs)
        if (!device_pointer(q, dev)) return BSC_E_INVALID;
    unsigned char* base = nullptr;
    int rc = scratch_address(&base);
    if (rc) return rc;

    Ctx c;  // a view on the scratch: owns nothing, frees nothing
    c.P = *p;
    c.device = dev;
    c.stream = static_cast<cudaStream_t>(stream);
    c.timing = false;
    c.use_graphs = false;
    c.fg_m = 0;
    c.r = reinterpret_cast<double*>(base + kOffWork);
    c.part = reinterpret_cast<double*>(base + kOffPart);
    c.Hd = reinterpret_cast<double*>(base + kOffHd);
    c.sc = reinterpret_cast<Scalars*>(base + kOffSc);
    c.ticket = reinterpret_cast<unsigned*>(base + kOffTicket);
    c.h_sc = &g_host_scalars;
    // the array keeps the previous call's ticket and scalars: start from zero
    if (cudaMemsetAsync(base + kOffSc, 0, kScratchBytes - kOffSc, c.stream) != cudaSuccess) {
        (void)cudaGetLastError();
        return BSC_E_CUDA;
    }
    *info = bsc_solve_info{};
    return csr_solve_device(&c, n, rowptr, col, val, b, x, info);
}

}  // extern "C"
