// Neighbour counting that allocates nothing.
//
// Some callers cannot call cudaMalloc at the moment they need an answer.  Examples:
// - a host program capturing a CUDA graph in global capture mode, where allocation
//   calls are prohibited until the capture ends;
// - a simulation engine that reserves all device memory from its own pool at start-up
//   and forbids allocations afterwards.
// nnap_neighbor_counts_noalloc serves them.  It runs the same wrap, cell-binning and
// neighbour kernels as the handle-based path, but every scratch buffer lives in the
// fixed array below.  That array is part of the library image: every GPU that loads the
// library holds it until the process exits.
//
// The array is shared by all calls.  The first call on each device looks up the
// array's device address (cudaGetSymbolAddress) with that device current.  Make that
// first call before any stream capture.  Calls whose work overlaps on the GPU race on
// the array.  Each call clears the parts that must start at zero.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>

#include "../../include/nnap_gb300.h"
#include "common.cuh"

namespace nnapgb {
__global__ void k_wrap_bin(const StructDev*, const int*, const double*, const int*, int, int, double*, float4*,
                           float4*, int*, int*, int*);
__global__ void k_scan_excl(const int*, int, int*);
__global__ void k_fill_cells(const int*, int, const int*, int*, int*);
__global__ void k_sort_cells(const int*, int, int*);
__global__ void k_neighbors(const StructDev*, const int*, const double*, const float4*, const float4*, const int*,
                            const int*, const int*, int, PairBufs, int*, int*);
}  // namespace nnapgb

using namespace nnapgb;

namespace {

constexpr int kNoAllocMaxAtoms = 16384;
constexpr int kNoAllocMaxCells = 16384;
constexpr size_t kNoAllocBytes = 2u << 20;  // 2 MiB

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// Byte offsets of the scratch regions for n atoms and c cells.
struct Carve {
    size_t sdev, status, sid, xw, xf, xlo, cell_of, cell_count, cell_fill, cell_start, cell_atoms, end;
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

void cross3(const double* u, const double* v, double* r) {
    r[0] = u[1] * v[2] - v[1] * u[2];
    r[1] = u[2] * v[0] - v[2] * u[0];
    r[2] = u[0] * v[1] - v[0] * u[1];
}

}  // namespace

extern "C" int nnap_neighbor_counts_noalloc(int natoms, const double* d_x, const int* d_type, int box_kind,
                                            const double* box, double rcut, int* d_counts, void* stream) {
    if (natoms < 0 || natoms > kNoAllocMaxAtoms) return NNAP_ERR_CAPACITY;
    if (!box || !(rcut > 0.0) || box_kind < 0 || box_kind > 2) return NNAP_ERR_ARG;
    if (natoms > 0 && (!d_x || !d_type || !d_counts)) return NNAP_ERR_ARG;
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

    // structure descriptor (same geometry rules as the handle-based path)
    StructDev s;
    std::memset(&s, 0, sizeof s);
    s.kind = box_kind;
    for (int d = 0; d < 3; ++d) { s.a[d] = box[d]; s.b[d] = box[3 + d]; s.c[d] = box[6 + d]; }
    if (box_kind == 0) s.a[1] = s.a[2] = s.b[0] = s.b[2] = s.c[0] = s.c[1] = 0.0;
    else if (box_kind == 1) s.a[1] = s.a[2] = s.b[2] = 0.0;
    cross3(s.b, s.c, s.bc);
    cross3(s.c, s.a, s.ca);
    cross3(s.a, s.b, s.ab);
    s.vol = (s.a[1] * s.b[2] - s.b[1] * s.a[2]) * s.c[0] + (s.a[2] * s.b[0] - s.b[2] * s.a[0]) * s.c[1] +
            (s.a[0] * s.b[1] - s.b[0] * s.a[1]) * s.c[2];
    if (!(s.vol > 0.0)) return NNAP_ERR_ARG;
    auto nrm = [](const double* v) { return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); };
    const double h[3] = {s.vol / nrm(s.bc), s.vol / nrm(s.ca), s.vol / nrm(s.ab)};
    double ext = 0.0;
    long long ncells = 1;
    for (int d = 0; d < 3; ++d) {
        s.nc[d] = std::max(1, (int)std::floor(h[d] / rcut));
        s.nc[d] = std::min(s.nc[d], 1024);
        s.R[d] = (int)std::floor(rcut * s.nc[d] / h[d] + 1e-6) + 1;
        if (s.R[d] > 64) return NNAP_ERR_ARG;
        ncells *= s.nc[d];
        ext += std::fabs(s.a[d]) + std::fabs(s.b[d]) + std::fabs(s.c[d]);
    }
    if (ncells > kNoAllocMaxCells) return NNAP_ERR_CAPACITY;
    for (int d = 0; d < 3; ++d) { s.fa[d] = (float)s.a[d]; s.fb[d] = (float)s.b[d]; s.fc[d] = (float)s.c[d]; }
    s.rc2 = rcut * rcut;
    const int Rm = std::max(s.R[0], std::max(s.R[1], s.R[2]));
    const double eps = 16.0 * (ext * (2 + Rm)) * std::ldexp(1.0, -24);
    const double margin = 2.0 * std::sqrt(3.0) * rcut * eps + 3.0 * eps * eps + 16.0 * rcut * rcut * std::ldexp(1.0, -24);
    s.rc2_hi = (float)(rcut * rcut + margin) * (1.0f + 1e-6f);
    s.a0 = 0;
    s.n = natoms;
    s.c0 = 0;

    const Carve k = carve(natoms, (size_t)ncells);
    cudaStream_t st = (cudaStream_t)stream;
    StructDev* sdev = reinterpret_cast<StructDev*>(base + k.sdev);
    int* status = reinterpret_cast<int*>(base + k.status);
    int* sid = reinterpret_cast<int*>(base + k.sid);
    double* xw = reinterpret_cast<double*>(base + k.xw);
    float4* xf = reinterpret_cast<float4*>(base + k.xf);
    float4* xlo = reinterpret_cast<float4*>(base + k.xlo);
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
        k_neighbors<<<(natoms + 3) / 4, 128, 0, st>>>(sdev, sid, xw, xf, xlo, cell_of, cell_start, cell_atoms, natoms,
                                                    P, status, status + 1);
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
