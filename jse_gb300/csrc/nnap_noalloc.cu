// Neighbour counting that allocates nothing.
//
// Some callers cannot call cudaMalloc at the moment they need an answer:
// - a simulation engine, or a framework's caching allocator, that reserves all device
//   memory for its own pool at start-up, so that a later cudaMalloc fails or takes
//   memory the engine has already promised elsewhere;
// - code in a latency-critical loop, where cudaMalloc and cudaFree synchronise the
//   device and stall the work of every other stream.
// nnap_neighbor_counts_noalloc serves them.  It runs the same wrap, cell-binning and
// neighbour kernels as the handle-based path, with the same box geometry and checks
// (struct_geometry), but every scratch buffer lives in the fixed array below.  That
// array is part of the library image: every GPU that loads the library holds it until
// the process exits.
//
// The array is shared by all calls.  The first call on each device looks up the
// array's device address (cudaGetSymbolAddress) with that device current; make that
// first call before any stream capture.  Calls whose work overlaps on the GPU race on
// the array.  Each call clears the parts that must start at zero.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>

#include "api_internal.hpp"

using namespace nnapgb;

namespace {

constexpr int kNoAllocMaxAtoms = 16384;
constexpr int kNoAllocMaxCells = 16384;
constexpr size_t kNoAllocBytes = 2u << 20;  // 2 MiB

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// Byte offsets of the scratch regions for n atoms and c cells.
struct Carve {
    size_t sdev, status, sid, xw, xf, xlo, xfc, xloc, cell_of, cell_count, cell_fill, cell_start, cell_atoms, end;
};
constexpr Carve carve(size_t n, size_t c) {
    Carve k{};
    size_t o = 0;
    k.sdev = o;       o = align256(o + sizeof(StructDev));
    k.status = o;     o = align256(o + 2 * sizeof(int));
    k.sid = o;        o = align256(o + n * sizeof(int));
    k.xw = o;         o = align256(o + 3 * n * sizeof(double));
    k.xf = o;         o = align256(o + n * sizeof(float4));
    k.xlo = o;        o = align256(o + n * sizeof(float4));
    k.xfc = o;        o = align256(o + n * sizeof(float4));
    k.xloc = o;       o = align256(o + n * sizeof(float4));
    k.cell_of = o;    o = align256(o + n * sizeof(int));
    k.cell_count = o; o = align256(o + c * sizeof(int));
    k.cell_fill = o;  o = align256(o + c * sizeof(int));
    k.cell_start = o; o = align256(o + (c + 1) * sizeof(int));
    k.cell_atoms = o; o = align256(o + n * sizeof(int));
    k.end = o;
    return k;
}
static_assert(carve(kNoAllocMaxAtoms, kNoAllocMaxCells).end <= kNoAllocBytes, "scratch array too small");

constexpr int kMaxDevices = 64;
unsigned char* g_scratch_ptr[kMaxDevices] = {nullptr};

}  // namespace

extern "C" int nnap_neighbor_counts_noalloc(int natoms, const double* d_x, const int* d_type, int box_kind,
                                            const double* box, double rcut, int* d_counts, void* stream) {
    // every check that needs no device comes first
    if (natoms < 0) return NNAP_ERR_ARG;
    if (natoms > kNoAllocMaxAtoms) return NNAP_ERR_CAPACITY;
    if (natoms > 0 && (!d_x || !d_type || !d_counts)) return NNAP_ERR_ARG;
    StructDev s;
    const int geo = struct_geometry(box_kind, box, rcut, natoms, s, nullptr);
    if (geo != NNAP_OK) return geo;
    const long long ncells = (long long)s.nc[0] * s.nc[1] * s.nc[2];
    if (ncells > kNoAllocMaxCells) return NNAP_ERR_CAPACITY;

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return NNAP_ERR_CUDA;
    }
    if (!g_scratch_ptr[dev]) {  // once per device, with that device current
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
            cudaGetLastError();
            return NNAP_ERR_CUDA;
        }
        g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
    }
    unsigned char* base = g_scratch_ptr[dev];

    const Carve k = carve(natoms, (size_t)ncells);
    cudaStream_t st = (cudaStream_t)stream;
    StructDev* sdev = reinterpret_cast<StructDev*>(base + k.sdev);
    int* status = reinterpret_cast<int*>(base + k.status);
    int* sid = reinterpret_cast<int*>(base + k.sid);
    double* xw = reinterpret_cast<double*>(base + k.xw);
    float4* xf = reinterpret_cast<float4*>(base + k.xf);
    float4* xlo = reinterpret_cast<float4*>(base + k.xlo);
    float4* xfc = reinterpret_cast<float4*>(base + k.xfc);
    float4* xloc = reinterpret_cast<float4*>(base + k.xloc);
    int* cell_of = reinterpret_cast<int*>(base + k.cell_of);
    int* cell_count = reinterpret_cast<int*>(base + k.cell_count);
    int* cell_fill = reinterpret_cast<int*>(base + k.cell_fill);
    int* cell_start = reinterpret_cast<int*>(base + k.cell_start);
    int* cell_atoms = reinterpret_cast<int*>(base + k.cell_atoms);

    cudaError_t e = cudaMemcpyAsync(sdev, &s, sizeof s, cudaMemcpyHostToDevice, st);
    // the parts that must start at zero: status words, structure ids, cell counters
    if (e == cudaSuccess) e = cudaMemsetAsync(status, 0, 2 * sizeof(int), st);
    if (e == cudaSuccess && natoms) e = cudaMemsetAsync(sid, 0, natoms * sizeof(int), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(cell_count, 0, ncells * sizeof(int), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(cell_fill, 0, ncells * sizeof(int), st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return NNAP_ERR_CUDA;
    }
    if (natoms > 0) {
        k_wrap_bin<<<(natoms + 255) / 256, 256, 0, st>>>(sdev, sid, d_x, d_type, natoms, INT_MAX, xw, xf, xlo,
                                                         cell_of, cell_count, status);
    }
    k_scan_excl<<<1, 1024, 0, st>>>(cell_count, (int)ncells, cell_start);
    if (natoms > 0) {
        k_fill_cells<<<(natoms + 255) / 256, 256, 0, st>>>(cell_of, natoms, cell_start, cell_fill, cell_atoms);
        k_sort_cells<<<((int)ncells * 32 + 255) / 256, 256, 0, st>>>(cell_start, (int)ncells, cell_atoms);
        PairBufs P;
        std::memset(&P, 0, sizeof P);
        P.M = 0;  // count only: no pair rows are written
        P.count = d_counts;
        k_cell_order<<<(natoms + 255) / 256, 256, 0, st>>>(cell_atoms, natoms, xf, xlo, xfc, xloc);
        k_neighbors<<<(natoms + 3) / 4, 128, 0, st>>>(sdev, sid, xw, xf, xlo, xfc, xloc, cell_of, cell_start, cell_atoms,
                                                    natoms, P, status, status + 1);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return NNAP_ERR_CUDA;
    int bits = 0;
    e = cudaMemcpyAsync(&bits, status, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return NNAP_ERR_CUDA;
    }
    if (bits & ERRBIT_BAD_TYPE) return NNAP_ERR_BAD_TYPE;
    return NNAP_OK;
}
