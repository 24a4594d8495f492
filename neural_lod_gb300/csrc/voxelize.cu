// Conservative surface voxelization: the triangle/voxel overlap test of cuda_voxelizer's
// voxelize_triangle (cuda_voxelizer/src/voxelize.cu:58-190) with glm 0.9.9.8 vector expressions
// and the fused multiply-adds that nvcc's default contraction puts into that kernel (the
// reference's build passes no -fmad flag).  Every operation is written with its rounding
// (__fmaf_rn / __fmul_rn / __fadd_rn / __fsub_rn / __fdiv_rn / __fsqrt_rn), so the voxel set is
// bit-exact with the reference kernel as built, and with the same arithmetic on the host:
//   per triangle  cross: fma(a.y, b.z, -(b.y*a.z)) ...; dot3: fma(a.z, b.z, fma(a.x, b.x, a.y*b.y));
//                 edge offsets: -1 * fma(n1, v_b, n0*v_a)
//   per voxel     n.p: fma(n.x, p.x, n.y*p.y) + n.z*p.z, but (n.x*p.x + n.y*p.y) + n.z*p.z in the
//                 first voxel of a row with an odd voxel count (the reference's x loop, unrolled by
//                 two, runs that voxel on its own); XY and YZ edge tests: fma(n0, p_a, n1*p_b) + d;
//                 ZX edge tests: fma(n1, p.x, n0*p.z) + d.
//
// Work split.  The reference runs one thread per triangle and loops over the triangle's
// candidate box, so one large triangle stalls its warp.  Here a warp stages 32 triangles in shared
// memory; triangles with at most `small_limit` candidate voxels are tested one per lane (a
// warp-converged loop of at most small_limit steps), larger ones one at a time by the whole warp,
// each lane taking every 32nd candidate.  Bits are set with one atomicOr per distinct word per
// warp step (lanes that hit the same word OR their masks first).
#include <cstdint>

#include "vox.h"

namespace nlod {
namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;
constexpr int kVoxThreads = 256;

// glm::min / glm::max / glm::clamp on floats (comparison forms)
__device__ __forceinline__ float gmin(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float gmax(float a, float b) { return (a < b) ? b : a; }
__device__ __forceinline__ float dot3(float a0, float a1, float a2, float b0, float b1, float b2) {
    return __fmaf_rn(a2, b2, __fmaf_rn(a0, b0, __fmul_rn(a1, b1)));
}

// Everything the per-voxel test of one triangle needs.
struct TriTest {
    float n[3], d1, d2;
    float ne[3][3][2];   // [plane XY/YZ/ZX][edge][2] projected edge normals
    float de[3][3];      // their offsets
    int32_t lo[3];       // candidate box (voxel indices)
    int32_t ext[3];      // its extent per axis
};

__device__ __forceinline__ void tri_setup(const float* T, const VoxFrame& f, TriTest& t) {
    float v[3][3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int i = 0; i < 3; ++i) v[k][i] = __fsub_rn(T[3 * k + i], f.bmin[i]);
    float e[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        e[0][i] = __fsub_rn(v[1][i], v[0][i]);
        e[1][i] = __fsub_rn(v[2][i], v[1][i]);
        e[2][i] = __fsub_rn(v[0][i], v[2][i]);
    }
    const float c0 = __fmaf_rn(e[0][1], e[1][2], -__fmul_rn(e[1][1], e[0][2]));
    const float c1 = __fmaf_rn(e[0][2], e[1][0], -__fmul_rn(e[1][2], e[0][0]));
    const float c2 = __fmaf_rn(e[0][0], e[1][1], -__fmul_rn(e[1][0], e[0][1]));
    const float inv_len = __fdiv_rn(1.0f, __fsqrt_rn(dot3(c0, c1, c2, c0, c1, c2)));
    t.n[0] = __fmul_rn(c0, inv_len);
    t.n[1] = __fmul_rn(c1, inv_len);
    t.n[2] = __fmul_rn(c2, inv_len);
    const float gm = (float)(f.grid - 1);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float wmin = gmin(v[0][i], gmin(v[1][i], v[2][i]));
        const float wmax = gmax(v[0][i], gmax(v[1][i], v[2][i]));
        const int32_t lo = (int32_t)gmin(gmax(__fdiv_rn(wmin, f.unit[i]), 0.0f), gm);
        const int32_t hi = (int32_t)gmin(gmax(__fdiv_rn(wmax, f.unit[i]), 0.0f), gm);
        t.lo[i] = lo;
        t.ext[i] = hi - lo + 1;
    }
    float cv[3], dc[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float c = (t.n[i] > 0.0f) ? f.unit[i] : 0.0f;
        cv[i] = __fsub_rn(c, v[0][i]);
        dc[i] = __fsub_rn(__fsub_rn(f.unit[i], c), v[0][i]);
    }
    t.d1 = dot3(t.n[0], t.n[1], t.n[2], cv[0], cv[1], cv[2]);
    t.d2 = dot3(t.n[0], t.n[1], t.n[2], dc[0], dc[1], dc[2]);
    // projections: XY (axes x,y; sign of n.z), YZ (y,z; n.x), ZX (z,x; n.y)
#pragma unroll
    for (int pl = 0; pl < 3; ++pl) {
        const int a = pl, b = (pl + 1) % 3, s = (pl + 2) % 3;
        const bool flip = t.n[s] < 0.0f;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            float n0 = __fmul_rn(-1.0f, e[k][b]), n1 = e[k][a];
            if (flip) {
                n0 = -n0;
                n1 = -n1;
            }
            t.ne[pl][k][0] = n0;
            t.ne[pl][k][1] = n1;
            t.de[pl][k] = __fadd_rn(__fadd_rn(__fmul_rn(-1.0f, __fmaf_rn(n1, v[k][b], __fmul_rn(n0, v[k][a]))), gmax(0.0f, __fmul_rn(f.unit[a], n0))),
                                    gmax(0.0f, __fmul_rn(f.unit[b], n1)));
        }
    }
}

// Overlap test of voxel (x, y, z) (grid indices) with the triangle.
__device__ __forceinline__ bool tri_hits(const TriTest& t, const VoxFrame& f, int32_t x, int32_t y, int32_t z) {
    const float p[3] = {__fmul_rn((float)x, f.unit[0]), __fmul_rn((float)y, f.unit[1]), __fmul_rn((float)z, f.unit[2])};
    // the reference build runs its x loop in pairs after one leading voxel when a row has an odd
    // voxel count; that leading voxel's plane dot product rounds all three products
    const bool lead = x == t.lo[0] && (t.ext[0] & 1);
    const float nx = lead ? __fmul_rn(t.n[0], p[0]) : 0.0f;
    const float nd = lead ? __fadd_rn(__fadd_rn(nx, __fmul_rn(t.n[1], p[1])), __fmul_rn(t.n[2], p[2]))
                          : __fadd_rn(__fmaf_rn(t.n[0], p[0], __fmul_rn(t.n[1], p[1])), __fmul_rn(t.n[2], p[2]));
    if (__fmul_rn(__fadd_rn(nd, t.d1), __fadd_rn(nd, t.d2)) > 0.0f) return false;
    bool ok = true;
#pragma unroll
    for (int pl = 0; pl < 3; ++pl) {
        const int a = pl, b = (pl + 1) % 3;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float n0 = t.ne[pl][k][0], n1 = t.ne[pl][k][1];
            const float s = pl == 2 ? __fmaf_rn(n1, p[b], __fmul_rn(n0, p[a])) : __fmaf_rn(n0, p[a], __fmul_rn(n1, p[b]));
            ok &= !(__fadd_rn(s, t.de[pl][k]) < 0.0f);
        }
    }
    return ok;
}

// Sets the bit of voxel (x, y, z) for every lane with hit; one atomicOr per distinct word.
// Must be called by all 32 lanes.
__device__ __forceinline__ void set_bits(uint32_t* __restrict__ bits, bool hit, uint32_t grid, int32_t x, int32_t y, int32_t z) {
    if (!__any_sync(kFull, hit)) return;
    const uint64_t loc = (uint64_t)x + (uint64_t)y * grid + (uint64_t)z * grid * grid;
    const uint32_t word = hit ? (uint32_t)(loc >> 5) : 0xFFFFFFFFu;
    const uint32_t mask = hit ? (1u << (31u - (uint32_t)(loc & 31u))) : 0u;
    const unsigned peers = __match_any_sync(kFull, word);
    const uint32_t v = __reduce_or_sync(peers, mask);
    if (hit && (int)(threadIdx.x & 31) == __ffs(peers) - 1) atomicOr(bits + word, v);
}

__global__ void __launch_bounds__(kVoxThreads) k_voxelize(const float* __restrict__ tris, uint64_t n, VoxFrame f,
                                                          uint32_t* __restrict__ bits, uint32_t small_limit) {
    __shared__ float stage[kVoxThreads / 32][32 * 9];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    float* st = stage[w];
    const uint64_t n_warps = (uint64_t)gridDim.x * (kVoxThreads / 32);
    for (uint64_t base = ((uint64_t)blockIdx.x * (kVoxThreads / 32) + w) * 32; base < n; base += n_warps * 32) {
        const uint32_t here = (uint32_t)((n - base) < 32 ? (n - base) : 32);
        // coalesced staging of 32 triangles
        const float* src = tris + base * 9;
        __syncwarp();
        for (uint32_t i = lane; i < here * 9; i += 32) st[i] = src[i];
        __syncwarp();
        const bool has = (uint32_t)lane < here;
        uint32_t my_cnt = 0;
        bool big = false;
        {
            TriTest t;
            tri_setup(st + 9 * (has ? lane : 0), f, t);
            const uint64_t cnt = has ? (uint64_t)t.ext[0] * (uint64_t)t.ext[1] * (uint64_t)t.ext[2] : 0;
            big = cnt > small_limit;
            my_cnt = big ? 0u : (uint32_t)cnt;
            const uint32_t steps = __reduce_max_sync(kFull, my_cnt);
            int32_t x = 0, y = 0, z = 0;
            for (uint32_t k = 0; k < steps; ++k) {
                const bool valid = k < my_cnt;
                const bool hit = valid && tri_hits(t, f, t.lo[0] + x, t.lo[1] + y, t.lo[2] + z);
                set_bits(bits, hit, f.grid, t.lo[0] + x, t.lo[1] + y, t.lo[2] + z);
                if (++x == t.ext[0]) {
                    x = 0;
                    if (++y == t.ext[1]) {
                        y = 0;
                        ++z;
                    }
                }
            }
        }
        unsigned big_mask = __ballot_sync(kFull, big);
        while (big_mask) {
            const int b = __ffs(big_mask) - 1;
            big_mask &= big_mask - 1;
            TriTest t;
            tri_setup(st + 9 * b, f, t);   // every lane, same triangle
            const int32_t nx = t.ext[0], ny = t.ext[1], nz = t.ext[2];
            // lane's first candidate and the 32-candidate step in mixed radix (nx, ny, nz)
            int32_t x = lane % nx, y = (lane / nx) % ny, z = lane / (nx * ny);
            const int32_t dx = 32 % nx, q = 32 / nx, dy = q % ny, dz = q / ny;
            const uint64_t total = (uint64_t)nx * (uint64_t)ny * (uint64_t)nz;
            for (uint64_t k = 0; k < total; k += 32) {
                const bool valid = z < nz;
                const bool hit = valid && tri_hits(t, f, t.lo[0] + x, t.lo[1] + y, t.lo[2] + z);
                set_bits(bits, hit, f.grid, t.lo[0] + x, t.lo[1] + y, t.lo[2] + z);
                x += dx;
                int32_t carry = x >= nx;
                x -= carry ? nx : 0;
                y += dy + carry;
                carry = y >= ny;
                y -= carry ? ny : 0;
                z += dz + carry;
            }
        }
    }
}

__device__ __forceinline__ uint32_t order_key(float v) {
    const uint32_t u = __float_as_uint(v);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__global__ void __launch_bounds__(256) k_mesh_bounds(const float* __restrict__ tris, uint64_t n_vertices, uint32_t* __restrict__ keys) {
    uint32_t mn[3] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu}, mx[3] = {0u, 0u, 0u};
    for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n_vertices; v += (uint64_t)gridDim.x * blockDim.x) {
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const uint32_t k = order_key(tris[3 * v + i]);
            mn[i] = min(mn[i], k);
            mx[i] = max(mx[i], k);
        }
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        mn[i] = __reduce_min_sync(kFull, mn[i]);
        mx[i] = __reduce_max_sync(kFull, mx[i]);
    }
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            atomicMin(keys + i, mn[i]);
            atomicMax(keys + 3 + i, mx[i]);
        }
    }
}

int sm_count() {
    static int count = [] {
        int dev = 0, c = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 148;
        return c;
    }();
    return count;
}

}  // namespace

cudaError_t launch_voxelize(const float* tris, uint64_t n, const VoxFrame& f, uint32_t* bits, uint32_t small_limit, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const uint64_t warps = (n + 31) / 32;
    const uint64_t want = (warps + kVoxThreads / 32 - 1) / (kVoxThreads / 32);
    const uint64_t cap = (uint64_t)sm_count() * 8;   // 8 resident 256-thread CTAs per SM
    const unsigned blocks = (unsigned)(want < cap ? want : cap);
    k_voxelize<<<blocks, kVoxThreads, 0, s>>>(tris, n, f, bits, small_limit);
    return cudaGetLastError();
}

cudaError_t launch_mesh_bounds(const float* tris, uint64_t n, uint32_t* keys, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const uint64_t nv = 3 * n;
    const uint64_t want = (nv + 255) / 256;
    const uint64_t cap = (uint64_t)sm_count() * 8;
    k_mesh_bounds<<<(unsigned)(want < cap ? want : cap), 256, 0, s>>>(tris, nv, keys);
    return cudaGetLastError();
}

}  // namespace nlod
