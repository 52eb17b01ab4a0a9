// Allocation-free broad phase: wg_broadphase_noalloc.
//
// Who needs it: a caller that must not allocate device memory -- for example a host process
// whose device memory is owned and budgeted by another runtime (a pooled allocator that
// forbids raw cudaMalloc/cudaFree), or a real-time loop that cannot afford the device-wide
// synchronisation that cudaMalloc/cudaFree imply. Such a caller can still hand over the sphere
// boxes in host memory and get the overlapping pairs back in host memory.
//
// How: the scratch that the regular broad phase allocates (boxes in device layout, grid keys,
// sort buffers, cell offsets, pair buffers, sort temporaries) lives in one file-scope
// __device__ array of fixed size. Every GPU that loads libwoogpu.so holds this array
// (WG_NOALLOC_SCRATCH_BYTES, about 13 MB) until the process exits. Sizes above
// WG_NOALLOC_MAX_SPHERES spheres or WG_NOALLOC_MAX_PAIRS pairs are rejected. Every call uses
// the same array, so two calls that overlap on the GPU (host threads calling it at the same
// time on one device) race and corrupt each other's result.
//
// The pair set is the one the collider computes for spheres: closed 3-axis overlap of the
// boxes and the mask test of Collider::mayCollide (pkg/dem/Collision.cpp:19-41).
#include <cub/cub.cuh>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "wg_internal.h"

#define WG_NOALLOC_MAX_SPHERES 32768
#define WG_NOALLOC_MAX_PAIRS 262144
#define WG_NOALLOC_MAX_CELLS (8 * WG_NOALLOC_MAX_SPHERES)

namespace wg_noalloc {

constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t NS = WG_NOALLOC_MAX_SPHERES, NP = WG_NOALLOC_MAX_PAIRS, NC = WG_NOALLOC_MAX_CELLS;
// scratch layout (byte offsets)
constexpr size_t O_RAWMN = 0;
constexpr size_t O_RAWMX = O_RAWMN + align256(sizeof(double) * 3 * NS);
constexpr size_t O_MASK = O_RAWMX + align256(sizeof(double) * 3 * NS);
constexpr size_t O_KEY = O_MASK + align256(sizeof(uint32_t) * NS);
constexpr size_t O_KEYS = O_KEY + align256(sizeof(uint32_t) * NS);
constexpr size_t O_VAL = O_KEYS + align256(sizeof(uint32_t) * NS);
constexpr size_t O_SID = O_VAL + align256(sizeof(int32_t) * NS);
constexpr size_t O_SMN = O_SID + align256(sizeof(int32_t) * NS);
constexpr size_t O_SMX = O_SMN + align256(sizeof(double) * 3 * NS);
constexpr size_t O_SMASK = O_SMX + align256(sizeof(double) * 3 * NS);
constexpr size_t O_OFF = O_SMASK + align256(sizeof(uint32_t) * NS);
constexpr size_t O_PAIRS = O_OFF + align256(sizeof(int32_t) * (NC + 1));
constexpr size_t O_PAIRSS = O_PAIRS + align256(sizeof(uint64_t) * NP);
constexpr size_t O_CNT = O_PAIRSS + align256(sizeof(uint64_t) * NP);
constexpr size_t O_RED = O_CNT + 256;
constexpr size_t O_TMP = O_RED + align256(sizeof(double) * 8 * 256);
constexpr size_t TMP_BYTES = size_t(4) << 20;
constexpr size_t SCRATCH_BYTES = O_TMP + TMP_BYTES;

}  // namespace wg_noalloc

// The scratch itself. Host code must not use this symbol as an address (it is a host-side
// stand-in); the device address is obtained with cudaGetSymbolAddress per device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[wg_noalloc::SCRATCH_BYTES];

namespace wg_noalloc {

static const int BS = 256;

// Per block: the lowest and highest box minimum per axis, the largest box extent, and the number
// of box components that are not finite (fmin/fmax skip NaN, so those are counted apart).
constexpr int NRED = 8;
__global__ void k_reduce_boxes(const double* __restrict__ mn, const double* __restrict__ mx, int n, double* __restrict__ partial) {
    __shared__ double s[NRED][BS];
    const double inf = __longlong_as_double(0x7ff0000000000000LL);
    double v[NRED] = {inf, inf, inf, -inf, -inf, -inf, 0., 0.};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        for (int k = 0; k < 3; k++) {
            const double a = mn[3 * i + k], b = mx[3 * i + k];
            if (!isfinite(a) || !isfinite(b)) {
                v[7] += 1.;
                continue;
            }
            v[k] = fmin(v[k], a);
            v[3 + k] = fmax(v[3 + k], a);
            v[6] = fmax(v[6], b - a);
        }
    }
    for (int q = 0; q < NRED; q++) s[q][threadIdx.x] = v[q];
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if (threadIdx.x < st) {
            for (int q = 0; q < 3; q++) s[q][threadIdx.x] = fmin(s[q][threadIdx.x], s[q][threadIdx.x + st]);
            for (int q = 3; q < 7; q++) s[q][threadIdx.x] = fmax(s[q][threadIdx.x], s[q][threadIdx.x + st]);
            s[7][threadIdx.x] += s[7][threadIdx.x + st];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int q = 0; q < NRED; q++) partial[blockIdx.x * NRED + q] = s[q][0];
}

__device__ __forceinline__ int cellCoord(double v, double o, double h, int n) {
    int ci = (int)floor((v - o) / h);
    return ci < 0 ? 0 : (ci >= n ? n - 1 : ci);
}

__global__ void k_keys(const double* __restrict__ mn, int n, double ox, double oy, double oz, double h, int nx, int ny, int nz,
                       uint32_t* __restrict__ key, int32_t* __restrict__ val) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int cx = cellCoord(mn[3 * i], ox, h, nx), cy = cellCoord(mn[3 * i + 1], oy, h, ny), cz = cellCoord(mn[3 * i + 2], oz, h, nz);
    key[i] = (uint32_t)(((int64_t)cz * ny + cy) * nx + cx);
    val[i] = i;
}

__global__ void k_offsets(const uint32_t* __restrict__ skey, int n, int64_t ncell, int32_t* __restrict__ off) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k > ncell) return;
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        const int64_t m = (lo + hi) >> 1;
        if (skey[m] < (uint32_t)k) lo = m + 1; else hi = m;
    }
    off[k] = (int32_t)lo;
}

__global__ void k_gather(const double* __restrict__ mn, const double* __restrict__ mx, const uint32_t* __restrict__ mask,
                         const int32_t* __restrict__ sid, int n, double* __restrict__ smn, double* __restrict__ smx,
                         uint32_t* __restrict__ smask) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int p = sid[i];
    for (int k = 0; k < 3; k++) {
        smn[3 * i + k] = mn[3 * p + k];
        smx[3 * i + k] = mx[3 * p + k];
    }
    smask[i] = mask[p];
}

__device__ __forceinline__ bool overlap(const double* a0, const double* a1, const double* b0, const double* b1) {
    return (a0[0] <= b1[0]) && (a1[0] >= b0[0]) && (a0[1] <= b1[1]) && (a1[1] >= b0[1]) && (a0[2] <= b1[2]) && (a1[2] >= b0[2]);
}

// half-shell sweep over the sorted cells (each pair met once)
__global__ void k_pairs(const int32_t* __restrict__ sid, const uint32_t* __restrict__ skey, const double* __restrict__ smn,
                        const double* __restrict__ smx, const uint32_t* __restrict__ smask, int n, int nx, int ny, int nz,
                        const int32_t* __restrict__ off, uint32_t lone, uint64_t* __restrict__ pairs, int64_t cap,
                        unsigned long long* __restrict__ counter) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t k = skey[i];
    const int cx = (int)(k % (uint32_t)nx), cy = (int)((k / (uint32_t)nx) % (uint32_t)ny), cz = (int)(k / ((uint32_t)nx * ny));
    const uint32_t m1 = smask[i];
    const int pi = sid[i];
    auto test = [&](int j) {
        const uint32_t mm = m1 & smask[j];
        if (mm != 0 && (mm & lone) == 0 && overlap(smn + 3 * i, smx + 3 * i, smn + 3 * j, smx + 3 * j)) {
            const int pj = sid[j];
            const int lo = pi < pj ? pi : pj, hi = pi < pj ? pj : pi;
            const unsigned long long idx = atomicAdd(counter, 1ull);
            if ((int64_t)idx < cap) pairs[idx] = ((uint64_t)(uint32_t)lo << 32) | (uint32_t)hi;
        }
    };
    {
        const int cx1 = cx + 1 < nx ? cx + 1 : cx;
        const int end = off[((int64_t)cz * ny + cy) * nx + cx1 + 1];
        for (int j = i + 1; j < end; j++) test(j);
    }
    const int DY[4] = {1, -1, 0, 1}, DZ[4] = {0, 1, 1, 1};
    for (int r = 0; r < 4; r++) {
        const int y = cy + DY[r], z = cz + DZ[r];
        if (y < 0 || y >= ny || z >= nz) continue;
        const int x0 = cx > 0 ? cx - 1 : 0, x1 = cx + 1 < nx ? cx + 1 : cx;
        const int64_t row = ((int64_t)z * ny + y) * nx;
        const int beg = off[row + x0], end = off[row + x1 + 1];
        for (int j = beg; j < end; j++) test(j);
    }
}

__global__ void k_split(const uint64_t* __restrict__ p, int64_t n, int32_t* __restrict__ lo, int32_t* __restrict__ hi) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    lo[i] = (int32_t)(p[i] >> 32);
    hi[i] = (int32_t)(p[i] & 0xffffffffu);
}

// one scratch address per device, resolved at the first call on that device with the device
// current (a cudaDeviceReset afterwards invalidates it: the library is not used across one)
static std::mutex g_mu;
static unsigned char* g_addr[64] = {nullptr};
static thread_local std::string g_err;

static int fail(int code, const std::string& m) {
    g_err = m;
    return code;
}

}  // namespace wg_noalloc

using namespace wg_noalloc;

extern "C" {

const char* wg_broadphase_noalloc_error(void) { return g_err.c_str(); }

int wg_broadphase_noalloc(int32_t n, const double* mn, const double* mx, const uint32_t* mask, uint32_t lone_mask, int64_t cap,
                          int32_t* id_lo, int32_t* id_hi, int64_t* n_pairs) {
    if (n_pairs) *n_pairs = 0;
    if (n < 0 || (n > 0 && (!mn || !mx || !mask)) || !n_pairs || cap < 0 || (cap > 0 && (!id_lo || !id_hi)))
        return fail(WG_ERR_ARG, "wg_broadphase_noalloc: invalid argument");
    if (n > WG_NOALLOC_MAX_SPHERES)
        return fail(WG_ERR_CAPACITY, "wg_broadphase_noalloc: more than " + std::to_string(WG_NOALLOC_MAX_SPHERES) +
                                         " spheres (the static scratch is sized for that many)");
    if (n == 0) return WG_OK;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return fail(WG_ERR_CUDA, "wg_broadphase_noalloc: no current device");
    unsigned char* base;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (!g_addr[dev]) {
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p) return fail(WG_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            g_addr[dev] = (unsigned char*)p;
        }
        base = g_addr[dev];
    }
    double* dmn = (double*)(base + O_RAWMN);
    double* dmx = (double*)(base + O_RAWMX);
    uint32_t* dmask = (uint32_t*)(base + O_MASK);
    uint32_t* key = (uint32_t*)(base + O_KEY);
    uint32_t* keys = (uint32_t*)(base + O_KEYS);
    int32_t* val = (int32_t*)(base + O_VAL);
    int32_t* sid = (int32_t*)(base + O_SID);
    double* smn = (double*)(base + O_SMN);
    double* smx = (double*)(base + O_SMX);
    uint32_t* smask = (uint32_t*)(base + O_SMASK);
    int32_t* off = (int32_t*)(base + O_OFF);
    uint64_t* pairs = (uint64_t*)(base + O_PAIRS);
    uint64_t* pairsS = (uint64_t*)(base + O_PAIRSS);
    unsigned long long* counter = (unsigned long long*)(base + O_CNT);
    double* red = (double*)(base + O_RED);
    void* tmp = (void*)(base + O_TMP);
    cudaStream_t st = 0;
#define NA_TRY(x)                                                                                         \
    do {                                                                                                  \
        cudaError_t _e = (x);                                                                             \
        if (_e != cudaSuccess) return fail(WG_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(_e)); \
    } while (0)
    NA_TRY(cudaMemcpy(dmn, mn, sizeof(double) * 3 * n, cudaMemcpyHostToDevice));
    NA_TRY(cudaMemcpy(dmx, mx, sizeof(double) * 3 * n, cudaMemcpyHostToDevice));
    NA_TRY(cudaMemcpy(dmask, mask, sizeof(uint32_t) * n, cudaMemcpyHostToDevice));
    // grid over the boxes: cell edge just above the largest box extent
    const int nb = std::min(256, (n + BS - 1) / BS);
    k_reduce_boxes<<<nb, BS, 0, st>>>(dmn, dmx, n, red);
    double hred[NRED * 256];
    NA_TRY(cudaMemcpy(hred, red, sizeof(double) * NRED * nb, cudaMemcpyDeviceToHost));
    double v[NRED] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY, 0., 0.};
    for (int b = 0; b < nb; b++) {
        for (int q = 0; q < 3; q++) v[q] = std::min(v[q], hred[NRED * b + q]);
        for (int q = 3; q < 7; q++) v[q] = std::max(v[q], hred[NRED * b + q]);
        v[7] += hred[NRED * b + 7];
    }
    if (v[7] != 0. || !(std::isfinite(v[0]) && std::isfinite(v[3]) && std::isfinite(v[6])))
        return fail(WG_ERR_ARG, "wg_broadphase_noalloc: boxes must be finite (NaN or infinite coordinate)");
    // cell edge: at least the largest box extent (so that the half shell sees every overlap) and
    // at least the widest spread over the cube root of the cell budget (so that the grid fits);
    // the dimensions are formed in double and clamped before they are multiplied
    double range = 0.;
    for (int q = 0; q < 3; q++) range = std::max(range, v[3 + q] - v[q]);
    double h = std::max(v[6] * (1 + 1e-9), range / std::cbrt((double)WG_NOALLOC_MAX_CELLS));
    if (!(h > 0.) || !std::isfinite(h)) h = 1.;  // every box is the same point: one cell
    int64_t dims[3];
    for (;;) {
        double prod = 1.;
        for (int q = 0; q < 3; q++) {
            const double d = std::min(std::floor((v[3 + q] - v[q]) / h) + 1., (double)WG_NOALLOC_MAX_CELLS);
            dims[q] = (int64_t)d;
            prod *= d;
        }
        if (prod <= (double)WG_NOALLOC_MAX_CELLS) break;
        h *= 1.25;
    }
    const int64_t ncell = dims[0] * dims[1] * dims[2];
    k_keys<<<(n + BS - 1) / BS, BS, 0, st>>>(dmn, n, v[0], v[1], v[2], h, (int)dims[0], (int)dims[1], (int)dims[2], key, val);
    int endBit = 1;
    while ((int64_t(1) << endBit) < ncell) endBit++;
    size_t tb = 0;
    NA_TRY(cub::DeviceRadixSort::SortPairs(nullptr, tb, key, keys, val, sid, n, 0, endBit, st));
    if (tb > TMP_BYTES) return fail(WG_ERR_CAPACITY, "wg_broadphase_noalloc: sort scratch too small");
    tb = TMP_BYTES;
    NA_TRY(cub::DeviceRadixSort::SortPairs(tmp, tb, key, keys, val, sid, n, 0, endBit, st));
    k_offsets<<<(unsigned)((ncell + 1 + BS - 1) / BS), BS, 0, st>>>(keys, n, ncell, off);
    k_gather<<<(n + BS - 1) / BS, BS, 0, st>>>(dmn, dmx, dmask, sid, n, smn, smx, smask);
    // the counter keeps the previous call's value: clear it
    NA_TRY(cudaMemsetAsync(counter, 0, sizeof(unsigned long long), st));
    k_pairs<<<(n + BS - 1) / BS, BS, 0, st>>>(sid, keys, smn, smx, smask, n, (int)dims[0], (int)dims[1], (int)dims[2], off,
                                              lone_mask, pairs, (int64_t)WG_NOALLOC_MAX_PAIRS, counter);
    unsigned long long cnt = 0;
    NA_TRY(cudaMemcpy(&cnt, counter, sizeof(cnt), cudaMemcpyDeviceToHost));
    *n_pairs = (int64_t)cnt;
    if (cnt > (unsigned long long)WG_NOALLOC_MAX_PAIRS)
        return fail(WG_ERR_CAPACITY, "wg_broadphase_noalloc: more than " + std::to_string(WG_NOALLOC_MAX_PAIRS) + " pairs");
    if ((int64_t)cnt > cap) return fail(WG_ERR_CAPACITY, "wg_broadphase_noalloc: output capacity too small");
    if (cnt > 0) {
        int idBits = 1;
        while ((int64_t(1) << idBits) < n) idBits++;
        tb = 0;
        NA_TRY(cub::DeviceRadixSort::SortKeys(nullptr, tb, pairs, pairsS, (int)cnt, 0, 32 + idBits, st));
        if (tb > TMP_BYTES) return fail(WG_ERR_CAPACITY, "wg_broadphase_noalloc: sort scratch too small");
        tb = TMP_BYTES;
        NA_TRY(cub::DeviceRadixSort::SortKeys(tmp, tb, pairs, pairsS, (int)cnt, 0, 32 + idBits, st));
        // split into the (now free) unsorted pair buffer viewed as two int32 arrays
        int32_t* lo = (int32_t*)pairs;
        int32_t* hi = lo + cnt;
        k_split<<<(unsigned)((cnt + BS - 1) / BS), BS, 0, st>>>(pairsS, (int64_t)cnt, lo, hi);
        NA_TRY(cudaMemcpy(id_lo, lo, sizeof(int32_t) * cnt, cudaMemcpyDeviceToHost));
        NA_TRY(cudaMemcpy(id_hi, hi, sizeof(int32_t) * cnt, cudaMemcpyDeviceToHost));
    }
    NA_TRY(cudaGetLastError());
#undef NA_TRY
    return WG_OK;
}
}
