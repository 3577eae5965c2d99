// mc_group.cu — GroupTriangles (model3d/bvh.go:118-217) on the device, the
// ordering step of SaveGroupedSTL (model3d/mesh.go:724-742).
//
// The reference sorts the triangles by bounding-box midpoint along each axis
// (sortBounders, bvh.go:219-255), then splits recursively: a node of n > 2
// triangles keeps the axis whose two halves (the first n/2 of that axis'
// order and the rest) have the smallest summed box area (bestSplitAxis,
// bvh.go:199-217), and stably partitions the two other axes' orders into the
// halves (splitBounders, bvh.go:158-197).  A node of one or two triangles is
// written in its x order (groupBounders, bvh.go:135-156).
//
// Here the recursion runs breadth first, one depth at a time, over three
// position-indexed arrays (one per axis) that hold every node's three orders
// side by side: node k of depth L covers the same positions in all three.
// Node sizes at one depth are floor or ceil of T / 2^L, so the host knows
// each depth's shape from T alone and picks its kernels:
//  * the three midpoint sorts: a stable LSD radix sort, 8 bits a pass, of
//    order-preserving 64-bit keys (ties keep the input order; a pass whose
//    digit is the same for every key is skipped);
//  * depths whose nodes exceed 1024 triangles: tile reductions of the half
//    boxes (shared, then global atomics on order-preserving keys; min and
//    max are exact in any order), one thread per node to pick the axis, and
//    a stable partition of the three orders through a global prefix sum;
//  * depths whose nodes hold 33..1024 triangles: one warp per node;
//  * the first depth whose nodes hold at most 32: one thread per node
//    finishes its subtree and writes the final order.
// Area arithmetic is float64 with no contraction, in boundsArea's order.

#include "mc_group.h"

#include <algorithm>
#include <vector>

namespace mcgpu {

namespace {

#define G_ADD __dadd_rn
#define G_SUB __dsub_rn
#define G_MUL __dmul_rn

constexpr int kThreads = 256;
constexpr int kPerThread = 16;
constexpr int kTile = kThreads * kPerThread;  // positions per CTA in the tiled kernels
#ifndef MC_GROUP_WARP_MAX
#define MC_GROUP_WARP_MAX 1024
#endif
constexpr int kWarpMax = MC_GROUP_WARP_MAX;   // largest node one warp splits
constexpr int kThreadMax = 32;                // largest node one thread finishes
// (node, half) segments one tile of a wide depth can touch: its halves hold
// at least kWarpMax / 2 triangles.
constexpr int kSlots = kTile / (kWarpMax / 2) + 2;
constexpr int kStack = 32;                    // finish-kernel stack entries (12 suffice for 32 triangles)

struct GBuf {
    void* p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        const size_t want = std::max<size_t>(bytes + bytes / 4, 256);
        cudaError_t e = cudaMalloc(&p, want);
        if (e == cudaSuccess) cap = want;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
    template <class T>
    T* as() const {
        return (T*)p;
    }
};

__device__ __forceinline__ double g_inf() { return __longlong_as_double(0x7ff0000000000000LL); }

// Order-preserving key of a float64: compares as the value does under `<`
// (-0 and +0 map to one key; no NaN reaches here).
__device__ __forceinline__ unsigned long long okey(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(G_ADD(v, 0.0));
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double odec(unsigned long long k) {
    return __longlong_as_double((long long)((k >> 63) ? (k & 0x7fffffffffffffffull) : ~k));
}

// boundsArea (bvh.go:289-292).
__device__ __forceinline__ double bounds_area(double x0, double y0, double z0, double x1, double y1, double z1) {
    const double dx = G_SUB(x1, x0), dy = G_SUB(y1, y0), dz = G_SUB(z1, z0);
    return G_MUL(2.0, G_ADD(G_MUL(dx, G_ADD(dy, dz)), G_MUL(dy, dz)));
}

// Node k of depth L of the halving tree over [0, T): first position and size.
__device__ __forceinline__ void gt_node(long long T, int L, long long k, long long* lo, long long* n) {
    long long l = 0, m = T;
    for (int d = L - 1; d >= 0; d--) {
        const long long h = m / 2;
        if ((k >> d) & 1) {
            l += h;
            m -= h;
        } else {
            m = h;
        }
    }
    *lo = l;
    *n = m;
}

// The depth-L node holding position p; its first position and size.
__device__ __forceinline__ long long gt_find(long long T, int L, long long p, long long* lo, long long* n) {
    long long l = 0, m = T, k = 0;
    for (int d = 0; d < L; d++) {
        const long long h = m / 2;
        if (p - l < h) {
            m = h;
            k = 2 * k;
        } else {
            l += h;
            m -= h;
            k = 2 * k + 1;
        }
    }
    *lo = l;
    *n = m;
    return k;
}

// ---------------------------------------------------------------- boxes

// Triangle.Min / Max (primitives.go:36-43) and the midpoint keys
// (Coord3D.Mid, the sort key of sortBounders).  Boxes are kept as
// order-preserving keys (okey): the reductions and comparisons of the
// splits then run on the integer pipes instead of the float64 pipe (1/60 of
// the float32 rate on this part); min and max commute with okey, and the
// areas decode them (-0 and +0 share a key: only the sign of a zero
// difference changes, which no comparison sees).
__global__ void k_gt_boxes(const double* __restrict__ verts, const int32_t* __restrict__ tris, long long T,
                           unsigned long long* __restrict__ box, unsigned long long* __restrict__ keys,
                           int32_t* __restrict__ vals) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < T; t += (long long)gridDim.x * blockDim.x) {
        double p[3][3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const long long i = tris ? (long long)tris[3 * t + k] : 3 * t + k;  // null: a triangle soup
#pragma unroll
            for (int c = 0; c < 3; c++) p[k][c] = verts[3 * i + c];
        }
#pragma unroll
        for (int c = 0; c < 3; c++) {
            double mn = p[1][c] < p[0][c] ? p[1][c] : p[0][c];
            mn = p[2][c] < mn ? p[2][c] : mn;
            double mx = p[1][c] > p[0][c] ? p[1][c] : p[0][c];
            mx = p[2][c] > mx ? p[2][c] : mx;
            box[6 * t + c] = okey(mn);
            box[6 * t + 3 + c] = okey(mx);
            keys[c * T + t] = okey(G_MUL(G_ADD(mn, mx), 0.5));
            vals[c * T + t] = (int32_t)t;
        }
    }
}

// ---------------------------------------------------------------- radix sort

struct RsPass {
    const unsigned long long* kin[3];
    const int32_t* vin[3];
    unsigned long long* kout[3];
    int32_t* vout[3];
    int active[3];
};

struct Act3 {
    int a[3];
};

// Lanes with the same digit, for warp-aggregated counting; lanes past the
// end get a value no digit has.
__device__ __forceinline__ unsigned digit_peers(bool ok, unsigned dig, int lane) {
    return __match_any_sync(0xffffffffu, ok ? dig : 256u + (unsigned)lane);
}

// All eight digit histograms of each axis' keys: hist[axis][digit][256].
__global__ void __launch_bounds__(kThreads) k_rs_hist(const unsigned long long* __restrict__ keys, long long T,
                                                      unsigned int* __restrict__ hist) {
    __shared__ unsigned int h[8 * 256];
    for (int i = threadIdx.x; i < 8 * 256; i += blockDim.x) h[i] = 0;
    __syncthreads();
    const int a = blockIdx.y, lane = threadIdx.x & 31;
    const unsigned long long* k = keys + (size_t)a * T;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long base = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < T; base += stride) {
        const long long i = base + lane;
        const bool ok = i < T;
        const unsigned long long v = ok ? k[i] : 0;
#pragma unroll
        for (int d = 0; d < 8; d++) {
            const unsigned dig = (unsigned)(v >> (8 * d)) & 255u;
            const unsigned peers = digit_peers(ok, dig, lane);
            if (ok && __ffs(peers) - 1 == lane) atomicAdd(&h[d * 256 + dig], (unsigned)__popc(peers));
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 8 * 256; i += blockDim.x)
        if (h[i]) atomicAdd(&hist[(size_t)a * 2048 + i], h[i]);
}

// Per-tile digit counts, digit-major: cnt[axis][digit][tile].
__global__ void __launch_bounds__(kThreads) k_rs_count(RsPass rp, long long T, int d, long long nb,
                                                       unsigned int* __restrict__ cnt) {
    const int a = blockIdx.y;
    if (!rp.active[a]) return;
    __shared__ unsigned int h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long t0 = (long long)blockIdx.x * kTile + (long long)warp * 32 * kPerThread;
    for (int r = 0; r < kPerThread; r++) {
        const long long i = t0 + r * 32 + lane;
        const bool ok = i < T;
        const unsigned dig = ok ? (unsigned)(rp.kin[a][i] >> (8 * d)) & 255u : 0u;
        const unsigned peers = digit_peers(ok, dig, lane);
        if (ok && __ffs(peers) - 1 == lane) atomicAdd(&h[dig], (unsigned)__popc(peers));
    }
    __syncthreads();
    cnt[((size_t)a * 256 + threadIdx.x) * nb + blockIdx.x] = h[threadIdx.x];
}

// Exclusive prefix sums of counts, in place.  One CTA of 1024 threads scans
// a chunk of up to kScanChunk counts (8 a thread); longer arrays are scanned
// chunk by chunk in parallel, then the chunk totals, then the offsets added.
constexpr int kScanE = 8;
constexpr long long kScanChunk = 1024LL * kScanE;

// Scans d[0, n) (n <= kScanChunk), adding `add`; returns the chunk's total.
__device__ unsigned cta_scan_chunk(unsigned int* __restrict__ d, long long n, unsigned add) {
    __shared__ unsigned int ws[32];
    __shared__ unsigned int total;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned v[kScanE], s = 0;
#pragma unroll
    for (int k = 0; k < kScanE; k++) {
        const long long i = (long long)threadIdx.x * kScanE + k;
        v[k] = i < n ? d[i] : 0u;
        s += v[k];
    }
    unsigned x = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[warp] = x;
    __syncthreads();
    if (warp == 0) {
        unsigned w = ws[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        ws[lane] = w;
        if (lane == 31) total = w;
    }
    __syncthreads();
    unsigned e = add + (warp ? ws[warp - 1] : 0u) + x - s;
#pragma unroll
    for (int k = 0; k < kScanE; k++) {
        const long long i = (long long)threadIdx.x * kScanE + k;
        if (i < n) d[i] = e;
        e += v[k];
    }
    const unsigned t = total;
    __syncthreads();  // ws and total are reused by the next call
    return t;
}

// n counts per axis (blockIdx.x), one CTA each, chunk after chunk.
__global__ void __launch_bounds__(1024) k_gt_scan(unsigned int* __restrict__ data, long long n, Act3 act) {
    if (!act.a[blockIdx.x]) return;
    unsigned int* dd = data + (size_t)blockIdx.x * n;
    unsigned carry = 0;
    for (long long base = 0; base < n; base += kScanChunk)
        carry += cta_scan_chunk(dd + base, min(kScanChunk, n - base), carry);
}

// Chunk c of axis blockIdx.y scanned on its own; its total to tot[axis][c].
__global__ void __launch_bounds__(1024) k_gt_scan_part(unsigned int* __restrict__ data, long long n, Act3 act,
                                                       unsigned int* __restrict__ tot, long long nchunk) {
    if (!act.a[blockIdx.y]) return;
    const long long base = (long long)blockIdx.x * kScanChunk;
    const unsigned t = cta_scan_chunk(data + (size_t)blockIdx.y * n + base, min(kScanChunk, n - base), 0u);
    if (threadIdx.x == 0) tot[(size_t)blockIdx.y * nchunk + blockIdx.x] = t;
}

__global__ void __launch_bounds__(1024) k_gt_scan_add(unsigned int* __restrict__ data, long long n, Act3 act,
                                                      const unsigned int* __restrict__ tot, long long nchunk) {
    if (!act.a[blockIdx.y]) return;
    const unsigned add = tot[(size_t)blockIdx.y * nchunk + blockIdx.x];
    unsigned int* d = data + (size_t)blockIdx.y * n + (long long)blockIdx.x * kScanChunk;
    const long long m = min(kScanChunk, n - (long long)blockIdx.x * kScanChunk);
    for (long long i = threadIdx.x; i < m; i += blockDim.x) d[i] += add;
}

// Stable scatter of one digit pass: warps take consecutive 512-key runs of
// the tile, lanes rank within a round by lane order.
__global__ void __launch_bounds__(kThreads) k_rs_scatter(RsPass rp, long long T, int d, long long nb,
                                                         const unsigned int* __restrict__ cnt) {
    const int a = blockIdx.y;
    if (!rp.active[a]) return;
    __shared__ unsigned int wh[kThreads / 32][256];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < (kThreads / 32) * 256; i += blockDim.x) (&wh[0][0])[i] = 0;
    __syncthreads();
    const long long t0 = (long long)blockIdx.x * kTile + (long long)warp * 32 * kPerThread;
    unsigned long long key[kPerThread];
    int32_t val[kPerThread];
#pragma unroll
    for (int r = 0; r < kPerThread; r++) {
        const long long i = t0 + r * 32 + lane;
        const bool ok = i < T;
        key[r] = ok ? rp.kin[a][i] : 0ull;
        val[r] = ok ? rp.vin[a][i] : 0;
        const unsigned dig = (unsigned)(key[r] >> (8 * d)) & 255u;
        const unsigned peers = digit_peers(ok, dig, lane);
        if (ok && __ffs(peers) - 1 == lane) wh[warp][dig] += (unsigned)__popc(peers);
        __syncwarp();
    }
    __syncthreads();
    {
        const int b = threadIdx.x;
        unsigned run = cnt[((size_t)a * 256 + b) * nb + blockIdx.x];
        for (int w = 0; w < kThreads / 32; w++) {
            const unsigned c = wh[w][b];
            wh[w][b] = run;
            run += c;
        }
    }
    __syncthreads();
    const unsigned lt = (1u << lane) - 1u;
#pragma unroll
    for (int r = 0; r < kPerThread; r++) {
        const long long i = t0 + r * 32 + lane;
        const bool ok = i < T;
        const unsigned dig = (unsigned)(key[r] >> (8 * d)) & 255u;
        const unsigned peers = digit_peers(ok, dig, lane);
        const unsigned pos = ok ? wh[warp][dig] + (unsigned)__popc(peers & lt) : 0u;
        __syncwarp();
        if (ok && __ffs(peers) - 1 == lane) wh[warp][dig] += (unsigned)__popc(peers);
        __syncwarp();
        if (ok) {
            rp.kout[a][pos] = key[r];
            rp.vout[a][pos] = val[r];
        }
    }
}

// ---------------------------------------------------------------- wide depths

// acc[node][axis][half][6]: min x y z, max x y z as order-preserving keys.
__device__ __forceinline__ size_t acc_at(long long key, int a) {
    return ((size_t)(key >> 1) * 3 + a) * 12 + (size_t)(key & 1) * 6;
}

__global__ void k_gt_acc_init(unsigned long long* __restrict__ acc, long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        acc[i] = (i % 6) < 3 ? ~0ull : 0ull;
}

// A triangle's box (min x y z, max x y z, as okeys) in three 16-byte loads.
__device__ __forceinline__ void load_box(const unsigned long long* __restrict__ box, int32_t t,
                                         unsigned long long b[6]) {
    const ulonglong2* q = reinterpret_cast<const ulonglong2*>(box + 6 * (size_t)t);
    const ulonglong2 u = q[0], v = q[1], w = q[2];
    b[0] = u.x;
    b[1] = u.y;
    b[2] = v.x;
    b[3] = v.y;
    b[4] = w.x;
    b[5] = w.y;
}

__device__ __forceinline__ void box_empty(unsigned long long b[6]) {
#pragma unroll
    for (int c = 0; c < 3; c++) {
        b[c] = ~0ull;
        b[3 + c] = 0ull;
    }
}

__device__ __forceinline__ void box_widen(unsigned long long b[6], const unsigned long long q[6]) {
#pragma unroll
    for (int c = 0; c < 3; c++) {
        b[c] = min(b[c], q[c]);
        b[3 + c] = max(b[3 + c], q[3 + c]);
    }
}

// boundsArea of a box of okeys.
__device__ __forceinline__ double key_area(const unsigned long long b[6]) {
    return bounds_area(odec(b[0]), odec(b[1]), odec(b[2]), odec(b[3]), odec(b[4]), odec(b[5]));
}

// multipleBoundsArea's boxes (bvh.go:257-287) of every node half, one axis'
// order per blockIdx.y.  A thread reduces 16 consecutive positions and
// flushes each half it met into the tile's shared slots.
__global__ void __launch_bounds__(kThreads) k_gt_reduce(const int32_t* __restrict__ ord,
                                                        const unsigned long long* __restrict__ box,
                                                        long long T, int L, unsigned long long* __restrict__ acc,
                                                        int* __restrict__ err) {
    const int a = blockIdx.y;
    const int32_t* o = ord + (size_t)a * T;
    __shared__ unsigned long long s[kSlots * 6];
    __shared__ long long key0_s;
    const long long p0 = (long long)blockIdx.x * kTile;
    for (int i = threadIdx.x; i < kSlots * 6; i += blockDim.x) s[i] = (i % 6) < 3 ? ~0ull : 0ull;
    if (threadIdx.x == 0) {
        long long lo, n;
        const long long k = gt_find(T, L, p0, &lo, &n);
        key0_s = 2 * k + ((p0 - lo) >= n / 2 ? 1 : 0);
    }
    __syncthreads();
    const long long key0 = key0_s;
    long long p = p0 + (long long)threadIdx.x * kPerThread;
    const long long pe = min(p + kPerThread, T);
    long long seg_end = -1, key = 0;
    unsigned long long bx[6];
    bool have = false;
    auto flush = [&]() {
        const long long sl = key - key0;
        if (sl < 0 || sl >= kSlots) {
            atomicOr(err, 1);
            return;
        }
#pragma unroll
        for (int c = 0; c < 3; c++) {
            atomicMin(&s[sl * 6 + c], bx[c]);
            atomicMax(&s[sl * 6 + 3 + c], bx[3 + c]);
        }
    };
    for (; p < pe; p++) {
        if (p >= seg_end) {
            if (have) flush();
            long long lo, n;
            const long long k = gt_find(T, L, p, &lo, &n);
            const long long h = n / 2;
            const int half = (p - lo) >= h ? 1 : 0;
            key = 2 * k + half;
            seg_end = half ? lo + n : lo + h;
            box_empty(bx);
            have = true;
        }
        unsigned long long b[6];
        load_box(box, o[p], b);
        box_widen(bx, b);
    }
    if (have) flush();
    __syncthreads();
    for (int i = threadIdx.x; i < kSlots * 6; i += blockDim.x) {
        const int sl = i / 6, c = i % 6;
        const unsigned long long v = s[i];
        if (c < 3 ? v != ~0ull : v != 0ull) {
            unsigned long long* g = acc + acc_at(key0 + sl, a) + c;
            if (c < 3) atomicMin(g, v);
            else atomicMax(g, v);
        }
    }
}

// bestSplitAxis (bvh.go:199-217) of every node of a wide depth.
__global__ void k_gt_axis(const unsigned long long* __restrict__ acc, long long NL, uint8_t* __restrict__ axis) {
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < NL; k += (long long)gridDim.x * blockDim.x) {
        int ax = 0;
        double best = 0;
        for (int a = 0; a < 3; a++) {
            const unsigned long long* q = acc + acc_at(2 * k, a);
            const double v = G_ADD(key_area(q), key_area(q + 6));
            if (a == 0 || v < best) {
                best = v;
                ax = a;
            }
        }
        axis[k] = (uint8_t)ax;
    }
}

// The split's flags (bvh.go:160-162): lower[t] = t is in its node's first
// half along the node's axis.
__global__ void k_gt_flag(const int32_t* __restrict__ ord, long long T, int L, const uint8_t* __restrict__ axis,
                          uint8_t* __restrict__ lower) {
    for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < T; p += (long long)gridDim.x * blockDim.x) {
        long long lo, n;
        const long long k = gt_find(T, L, p, &lo, &n);
        lower[ord[(size_t)axis[k] * T + p]] = (p - lo) < n / 2 ? 1 : 0;
    }
}

// Lower-half flags per tile of each axis' order: pcnt[axis][tile].
__global__ void __launch_bounds__(kThreads) k_gt_pcount(const int32_t* __restrict__ ord, const uint8_t* __restrict__ lower,
                                                        long long T, long long nb, unsigned int* __restrict__ pcnt) {
    const int a = blockIdx.y;
    __shared__ unsigned int ws[kThreads / 32];
    const long long p0 = (long long)blockIdx.x * kTile + (long long)threadIdx.x * kPerThread;
    unsigned c = 0;
    for (int r = 0; r < kPerThread; r++) {
        const long long p = p0 + r;
        if (p < T) c += lower[ord[(size_t)a * T + p]];
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned t = 0;
        for (int w = 0; w < kThreads / 32; w++) t += ws[w];
        pcnt[(size_t)a * nb + blockIdx.x] = t;
    }
}

// splitBounders' stable partition (bvh.go:164-184) of all three orders:
// a lower triangle goes to lo + (lower ones before it in the node), an upper
// one to lo + n/2 + (upper ones before it).  `before` holds, per node, the
// lower triangles of the nodes left of it (sum of their n/2).
__global__ void __launch_bounds__(kThreads) k_gt_pscatter(const int32_t* __restrict__ oin, int32_t* __restrict__ oout,
                                                          const uint8_t* __restrict__ lower, long long T, int L,
                                                          const unsigned int* __restrict__ pcnt, long long nb,
                                                          const long long* __restrict__ before) {
    const int a = blockIdx.y;
    const int32_t* o = oin + (size_t)a * T;
    int32_t* w = oout + (size_t)a * T;
    __shared__ unsigned int ws[kThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long p0 = (long long)blockIdx.x * kTile + (long long)threadIdx.x * kPerThread;
    int32_t t[kPerThread];
    unsigned fl = 0, s = 0;
#pragma unroll
    for (int r = 0; r < kPerThread; r++) {
        const long long p = p0 + r;
        t[r] = p < T ? o[p] : 0;
        const unsigned f = p < T ? lower[t[r]] : 0u;
        fl |= f << r;
        s += f;
    }
    unsigned x = s;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x += y;
    }
    if (lane == 31) ws[warp] = x;
    __syncthreads();
    unsigned wpre = 0;
    for (int k = 0; k < warp; k++) wpre += ws[k];
    long long G = (long long)pcnt[(size_t)a * nb + blockIdx.x] + wpre + x - s;  // lower ones before p0
    long long node_end = -1, lo = 0, n = 0, LB = 0;
    for (int r = 0; r < kPerThread; r++) {
        const long long p = p0 + r;
        if (p >= T) break;
        if (p >= node_end) {
            const long long k = gt_find(T, L, p, &lo, &n);
            node_end = lo + n;
            LB = before[k];
        }
        const long long rl = G - LB;  // lower ones in [lo, p)
        const bool f = (fl >> r) & 1u;
        w[f ? lo + rl : lo + n / 2 + (p - lo - rl)] = t[r];
        G += f ? 1 : 0;
    }
}

// ---------------------------------------------------------------- warp depths

__device__ __forceinline__ void box_warp_reduce(unsigned long long b[6]) {
#pragma unroll
    for (int o = 16; o; o >>= 1) {
#pragma unroll
        for (int c = 0; c < 3; c++) {
            b[c] = min(b[c], __shfl_xor_sync(0xffffffffu, b[c], o));
            b[3 + c] = max(b[3 + c], __shfl_xor_sync(0xffffffffu, b[3 + c], o));
        }
    }
}

// One warp per node of 33..1024 triangles: axis choice, flags, and the
// stable partition of all three orders (ballot ranks) into oout.  Lanes take
// four positions a round, loads first, for memory-level parallelism.
__global__ void __launch_bounds__(kThreads) k_gt_warp(const int32_t* __restrict__ oin, int32_t* __restrict__ oout,
                                                      const unsigned long long* __restrict__ box,
                                                      uint8_t* __restrict__ lower, long long T, int L, long long NL) {
    constexpr int U = 4;
    const int lane = threadIdx.x & 31;
    const long long k = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (k >= NL) return;  // warp-uniform
    long long lo, n;
    gt_node(T, L, k, &lo, &n);
    const int m = (int)n, h = m / 2;
    int ax = 0;
    double best = 0;
    for (int a = 0; a < 3; a++) {
        const int32_t* o = oin + (size_t)a * T + lo;
        unsigned long long b0[6], b1[6];
        box_empty(b0);
        box_empty(b1);
        for (int i0 = lane; i0 < m; i0 += 32 * U) {
            int32_t t[U];
#pragma unroll
            for (int u = 0; u < U; u++) t[u] = i0 + 32 * u < m ? o[i0 + 32 * u] : -1;
            unsigned long long q[U][6];
#pragma unroll
            for (int u = 0; u < U; u++)
                if (t[u] >= 0) load_box(box, t[u], q[u]);
#pragma unroll
            for (int u = 0; u < U; u++) {
                if (t[u] < 0) continue;
                if (i0 + 32 * u < h) box_widen(b0, q[u]);
                else box_widen(b1, q[u]);
            }
        }
        box_warp_reduce(b0);
        box_warp_reduce(b1);
        const double v = G_ADD(key_area(b0), key_area(b1));
        if (a == 0 || v < best) {
            best = v;
            ax = a;
        }
    }
    for (int i = lane; i < m; i += 32) lower[oin[(size_t)ax * T + lo + i]] = i < h ? 1 : 0;
    __syncwarp();
    const unsigned lt = (1u << lane) - 1u;
    for (int a = 0; a < 3; a++) {
        const int32_t* o = oin + (size_t)a * T + lo;
        int32_t* w = oout + (size_t)a * T + lo;
        int cl = 0, cu = 0;
        for (int base = 0; base < m; base += 32 * U) {
            int32_t t[U];
            bool f[U];
#pragma unroll
            for (int u = 0; u < U; u++) t[u] = base + 32 * u + lane < m ? o[base + 32 * u + lane] : -1;
#pragma unroll
            for (int u = 0; u < U; u++) f[u] = t[u] >= 0 && lower[t[u]];
#pragma unroll
            for (int u = 0; u < U; u++) {
                const bool ok = t[u] >= 0;
                const unsigned bl = __ballot_sync(0xffffffffu, f[u]), bv = __ballot_sync(0xffffffffu, ok);
                if (ok) w[f[u] ? cl + __popc(bl & lt) : h + cu + __popc(bv & ~bl & lt)] = t[u];
                cl += __popc(bl);
                cu += __popc(bv & ~bl);
            }
        }
    }
}

// ---------------------------------------------------------------- finish

constexpr int kFinishThreads = 128;

// multipleBoundsArea (bvh.go:257-287) of n local items.
__device__ double local_area(const unsigned long long* __restrict__ box, const int32_t* id, const uint8_t* s, int n) {
    unsigned long long b[6];
    load_box(box, id[s[0]], b);
    for (int i = 1; i < n; i++) {
        unsigned long long q[6];
        load_box(box, id[s[i]], q);
        box_widen(b, q);
    }
    return key_area(b);
}

// One thread per node of at most 32 triangles: the rest of groupBounders
// (bvh.go:135-156) depth first, writing the final order of its positions.
// (Boxes staged in shared memory measured slower: 48 KB per 32 threads
// leaves four warps an SM.)
__global__ void __launch_bounds__(kFinishThreads) k_gt_finish(const int32_t* __restrict__ oin,
                                                              const unsigned long long* __restrict__ box,
                                                              int32_t* __restrict__ loc,
                                                              long long T, int L, long long NL,
                                                              int32_t* __restrict__ order, int* __restrict__ err) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= NL) return;
    long long lo, n;
    gt_node(T, L, k, &lo, &n);
    if (n > kThreadMax || n < 1) {
        atomicOr(err, 2);
        return;
    }
    const int m = (int)n;
    int32_t id[kThreadMax];
    uint8_t s[3][kThreadMax], tmp[kThreadMax];
    for (int j = 0; j < m; j++) {
        id[j] = oin[lo + j];
        loc[id[j]] = j;
        s[0][j] = (uint8_t)j;
    }
    for (int a = 1; a < 3; a++)
        for (int j = 0; j < m; j++) s[a][j] = (uint8_t)loc[oin[(size_t)a * T + lo + j]];
    int stk[kStack];
    int sp = 0;
    stk[sp++] = 0;
    stk[sp++] = m;
    while (sp > 0) {
        const int c = stk[--sp];
        const int l = stk[--sp];
        if (c <= 2) {
            for (int i = 0; i < c; i++) order[lo + l + i] = id[s[0][l + i]];
            continue;
        }
        const int h = c / 2;
        int ax = 0;
        double best = 0;
        for (int a = 0; a < 3; a++) {
            const double v = G_ADD(local_area(box, id, s[a] + l, h), local_area(box, id, s[a] + l + h, c - h));
            if (a == 0 || v < best) {
                best = v;
                ax = a;
            }
        }
        unsigned low = 0;
        for (int i = 0; i < h; i++) low |= 1u << s[ax][l + i];
        for (int a = 0; a < 3; a++) {
            if (a == ax) continue;
            int k0 = 0, k1 = 0;
            for (int i = 0; i < c; i++) {
                const uint8_t x = s[a][l + i];
                if ((low >> x) & 1u) s[a][l + k0++] = x;
                else tmp[k1++] = x;
            }
            for (int i = 0; i < k1; i++) s[a][l + k0 + i] = tmp[i];
        }
        if (sp + 4 > kStack) {
            atomicOr(err, 4);
            return;
        }
        stk[sp++] = l + h;
        stk[sp++] = c - h;
        stk[sp++] = l;
        stk[sp++] = h;
    }
}

}  // namespace

struct GroupScratch {
    GBuf box, keys[2], vals[2], hist, cnt, lower, acc, axis, before, pcnt, loc, err, stot;
    ~GroupScratch() {
        for (GBuf* b : {&box, &keys[0], &keys[1], &vals[0], &vals[1], &hist, &cnt, &lower, &acc, &axis, &before,
                        &pcnt, &loc, &err, &stot})
            b->release();
    }
};

GroupScratch* group_scratch_new() { return new GroupScratch(); }

namespace {

// Exclusive scan of n counts for each active axis (data: 3 x n).
cudaError_t scan3(GroupScratch* g, unsigned int* data, long long n, Act3 act, cudaStream_t st) {
    if (n <= kScanChunk) {
        k_gt_scan<<<3, 1024, 0, st>>>(data, n, act);
        return cudaGetLastError();
    }
    const long long nchunk = (n + kScanChunk - 1) / kScanChunk;
    cudaError_t e = g->stot.ensure((size_t)3 * nchunk * 4);
    if (e != cudaSuccess) return e;
    k_gt_scan_part<<<dim3((unsigned)nchunk, 3), 1024, 0, st>>>(data, n, act, g->stot.as<unsigned int>(), nchunk);
    k_gt_scan<<<3, 1024, 0, st>>>(g->stot.as<unsigned int>(), nchunk, act);
    k_gt_scan_add<<<dim3((unsigned)nchunk, 3), 1024, 0, st>>>(data, n, act, g->stot.as<unsigned int>(), nchunk);
    return cudaGetLastError();
}

}  // namespace
void group_scratch_free(GroupScratch* g) { delete g; }

cudaError_t group_triangles_device(GroupScratch* g, const double* verts, const int32_t* tris, long long T,
                                   int32_t* order, cudaStream_t st, int sm_count, bool* internal_error) {
#define GK(x)                                \
    do {                                     \
        const cudaError_t e_ = (x);          \
        if (e_ != cudaSuccess) return e_;    \
    } while (0)
    *internal_error = false;
    if (T <= 0) return cudaSuccess;
    const long long nb = (T + kTile - 1) / kTile;
    const size_t t8 = (size_t)T * 8, t4 = (size_t)T * 4;
    GK(g->box.ensure(t8 * 6));
    for (int i = 0; i < 2; i++) {
        GK(g->keys[i].ensure(3 * t8));
        GK(g->vals[i].ensure(3 * t4));
    }
    GK(g->hist.ensure(3 * 2048 * 4));
    GK(g->cnt.ensure((size_t)3 * 256 * nb * 4));
    GK(g->pcnt.ensure((size_t)3 * nb * 4));
    GK(g->lower.ensure((size_t)T));
    GK(g->loc.ensure(t4));
    GK(g->err.ensure(4));
    GK(cudaMemsetAsync(g->err.p, 0, 4, st));
    int* err = g->err.as<int>();
    const int grid_t = (int)std::min<long long>((T + kThreads - 1) / kThreads, (long long)sm_count * 16);

    // Boxes, midpoint keys and the three stable sorts.
    k_gt_boxes<<<grid_t, kThreads, 0, st>>>(verts, tris, T, g->box.as<unsigned long long>(), g->keys[0].as<unsigned long long>(),
                                            g->vals[0].as<int32_t>());
    GK(cudaGetLastError());
    GK(cudaMemsetAsync(g->hist.p, 0, 3 * 2048 * 4, st));
    k_rs_hist<<<dim3((unsigned)std::min<long long>(nb, (long long)sm_count * 4), 3), kThreads, 0, st>>>(
        g->keys[0].as<unsigned long long>(), T, g->hist.as<unsigned int>());
    GK(cudaGetLastError());
    std::vector<unsigned int> hh(3 * 2048);
    GK(cudaMemcpyAsync(hh.data(), g->hist.p, hh.size() * 4, cudaMemcpyDeviceToHost, st));
    GK(cudaStreamSynchronize(st));
    int cur[3] = {0, 0, 0};
    for (int d = 0; d < 8; d++) {
        RsPass rp{};
        Act3 act{};
        bool any = false;
        for (int a = 0; a < 3; a++) {
            bool trivial = false;
            for (int b = 0; b < 256; b++) trivial |= hh[(size_t)a * 2048 + d * 256 + b] == (unsigned)T;
            rp.active[a] = act.a[a] = trivial ? 0 : 1;
            any |= !trivial;
            rp.kin[a] = g->keys[cur[a]].as<unsigned long long>() + (size_t)a * T;
            rp.vin[a] = g->vals[cur[a]].as<int32_t>() + (size_t)a * T;
            rp.kout[a] = g->keys[cur[a] ^ 1].as<unsigned long long>() + (size_t)a * T;
            rp.vout[a] = g->vals[cur[a] ^ 1].as<int32_t>() + (size_t)a * T;
        }
        if (!any) continue;
        k_rs_count<<<dim3((unsigned)nb, 3), kThreads, 0, st>>>(rp, T, d, nb, g->cnt.as<unsigned int>());
        GK(cudaGetLastError());
        GK(scan3(g, g->cnt.as<unsigned int>(), 256 * nb, act, st));
        k_rs_scatter<<<dim3((unsigned)nb, 3), kThreads, 0, st>>>(rp, T, d, nb, g->cnt.as<unsigned int>());
        GK(cudaGetLastError());
        for (int a = 0; a < 3; a++) cur[a] ^= act.a[a];
    }
    for (int a = 0; a < 3; a++)
        if (cur[a])
            GK(cudaMemcpyAsync(g->vals[0].as<int32_t>() + (size_t)a * T, g->vals[1].as<int32_t>() + (size_t)a * T, t4,
                               cudaMemcpyDeviceToDevice, st));

    // Per wide depth, the lower triangles left of each node (host: node
    // sizes depend on T alone).
    std::vector<long long> before, sizes{T};
    std::vector<size_t> before_at;
    for (int L = 0; (T + (1LL << L) - 1) >> L > kWarpMax; L++) {
        before_at.push_back(before.size());
        long long run = 0;
        std::vector<long long> next;
        next.reserve(sizes.size() * 2);
        for (long long s : sizes) {
            before.push_back(run);
            run += s / 2;
            next.push_back(s / 2);
            next.push_back(s - s / 2);
        }
        sizes.swap(next);
    }
    if (!before.empty()) {
        GK(g->before.ensure(before.size() * 8));
        GK(cudaMemcpyAsync(g->before.p, before.data(), before.size() * 8, cudaMemcpyHostToDevice, st));
        // `before` is pageable: the copy has read it when the call returns.
    }

    int32_t* oin = g->vals[0].as<int32_t>();
    int32_t* oout = g->vals[1].as<int32_t>();
    for (int L = 0;; L++) {
        const long long NL = 1LL << L;
        const long long nmax = (T + NL - 1) / NL;
        if (nmax <= kThreadMax) {
            k_gt_finish<<<(unsigned)((NL + kFinishThreads - 1) / kFinishThreads), kFinishThreads, 0, st>>>(
                oin, g->box.as<unsigned long long>(), g->loc.as<int32_t>(), T, L, NL, order, err);
            GK(cudaGetLastError());
            break;
        }
        if (nmax > kWarpMax) {
            GK(g->acc.ensure((size_t)NL * 36 * 8));
            GK(g->axis.ensure((size_t)NL));
            unsigned long long* acc = g->acc.as<unsigned long long>();
            const int ga = (int)std::min<long long>((NL * 36 + 255) / 256, (long long)sm_count * 16);
            k_gt_acc_init<<<ga, 256, 0, st>>>(acc, NL * 36);
            k_gt_reduce<<<dim3((unsigned)nb, 3), kThreads, 0, st>>>(oin, g->box.as<unsigned long long>(), T, L, acc, err);
            k_gt_axis<<<(unsigned)((NL + 255) / 256), 256, 0, st>>>(acc, NL, g->axis.as<uint8_t>());
            k_gt_flag<<<grid_t, kThreads, 0, st>>>(oin, T, L, g->axis.as<uint8_t>(), g->lower.as<uint8_t>());
            k_gt_pcount<<<dim3((unsigned)nb, 3), kThreads, 0, st>>>(oin, g->lower.as<uint8_t>(), T, nb,
                                                                     g->pcnt.as<unsigned int>());
            GK(scan3(g, g->pcnt.as<unsigned int>(), nb, Act3{{1, 1, 1}}, st));
            k_gt_pscatter<<<dim3((unsigned)nb, 3), kThreads, 0, st>>>(oin, oout, g->lower.as<uint8_t>(), T, L,
                                                                       g->pcnt.as<unsigned int>(), nb,
                                                                       g->before.as<long long>() + before_at[L]);
            GK(cudaGetLastError());
        } else {
            k_gt_warp<<<(unsigned)((NL * 32 + kThreads - 1) / kThreads), kThreads, 0, st>>>(
                oin, oout, g->box.as<unsigned long long>(), g->lower.as<uint8_t>(), T, L, NL);
            GK(cudaGetLastError());
        }
        std::swap(oin, oout);
    }
    int herr = 0;
    GK(cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, st));
    GK(cudaStreamSynchronize(st));
    *internal_error = herr != 0;
    return cudaSuccess;
#undef GK
}

}  // namespace mcgpu
