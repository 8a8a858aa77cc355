// Shared device-side definitions for the NNAP GB300 kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace nnapgb {

constexpr int kMaxTypes = 16;      // species supported per model
constexpr int kImgBias = 512;      // image components are packed as 10-bit biased fields

// Error bits raised by kernels into a device word and reported by the host.
enum : int {
    ERRBIT_CAPACITY = 1,    // a neighbour row overflowed its capacity
    ERRBIT_BAD_TYPE = 2,    // species outside 1..ntypes
    ERRBIT_NO_MIRROR = 4,   // a pair had no mirrored entry (asymmetric list)
    ERRBIT_CELLS = 8,       // an atom fell outside its structure's cell grid
    ERRBIT_TIMEOUT = 16     // a bounded device-side wait gave up
};

// One periodic structure of a batch, as the device sees it.
struct StructDev {
    double a[3], b[3], c[3];      // box rows (zeroed where the box kind ignores them)
    double bc[3], ca[3], ab[3];   // b x c, c x a, a x b (general prism)
    double vol;                   // a . (b x c)
    double rc2;                   // largest cutoff squared
    float fa[3], fb[3], fc[3];    // float box rows for the candidate screen
    float rc2_hi;                 // float screen bound (rc^2 plus rounding margin)
    float la[3], lb[3], lc[3];    // low parts of the box rows: a = fa + la to ~48 bits
    float iv[3][3];               // rows b x c, c x a, a x b over the volume: direct coordinates
    float smin2;                  // squared smallest singular value of the box matrix (0: unknown)
    int kind;                     // 0 orthogonal, 1 LAMMPS lower-triangular, 2 general prism
    int a0, n;                    // atom range in the batch
    int c0;                       // first cell of this structure in the global cell arrays
    int nc[3];                    // cells along a, b, c
    int R[3];                     // cell offsets searched along a, b, c
};

__host__ __device__ inline uint32_t pack_img(int na, int nb, int nc) {
    return ((uint32_t)(na + kImgBias) << 20) | ((uint32_t)(nb + kImgBias) << 10) | (uint32_t)(nc + kImgBias);
}
__host__ __device__ inline void unpack_img(uint32_t p, int& na, int& nb, int& nc) {
    na = (int)((p >> 20) & 1023u) - kImgBias;
    nb = (int)((p >> 10) & 1023u) - kImgBias;
    nc = (int)(p & 1023u) - kImgBias;
}
__host__ __device__ inline uint64_t pair_key(int j, uint32_t img) { return ((uint64_t)(uint32_t)j << 32) | img; }

// Device buffers of one evaluation (all owned by the handle; see nnap_api.cu).
constexpr int kLmpSumThreads = 256;  // threads of the LAMMPS global-virial sum

struct PairBufs {
    int M;                 // neighbour capacity per atom (row stride)
    uint64_t* key;         // [n*M] (j << 32) | packed image
    float4* dx;            // [n*M] (dx, dy, dz, bits of type_j)
    float4* dxlo;          // [n*M] low parts: dx = hi + lo to ~48 bits (NEP ZBL reads them), or NULL
    int* rev;              // [n*M] flat index of the mirrored entry
    float4* g;             // [n*M] pair gradient -dE_i/d(x_j - x_i)
    uint16_t* grp;         // [n*M] cell-offset group of the entry (rows are sorted by group, then j)
    int* count;            // [n] true neighbour count (may exceed M on overflow)
    int* gstart;           // [n][GS] row position where each cell-offset group starts (GS = 0: not kept)
    int GS;                // groups per atom + 1 (largest offset count of the batch + 1), or 0
};

}  // namespace nnapgb
