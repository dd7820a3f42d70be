// Welded Marching Cubes (MESH_ALG_MC_WELDED): one vertex per crossed lattice
// edge, from the per-cell mesh and its per-vertex edge keys.
//
// The expansion writes, beside every vertex of the ordinary (per-cell) mesh,
// its lattice edge and whether the emitting cell is the first cell of the
// emission order that meets that edge (Plan::vkey).  Because every crossed edge
// of a cell carries a vertex of that cell (the case tables place one on each),
// the first cell to meet an edge is the smallest cell containing it, and the
// welded mesh is:
//   vertices: the owned vertices, in order (a scan of the ownership flags);
//   faces: the ordinary faces with each vertex replaced by its edge's owned one
//          (a hash table from edge key to welded id).
// Four launches: per-block counts, one CTA scanning them, placement + hash
// insertion, face remapping.  Probing is bounded by the table size; a missing
// or duplicate key sets ERR_BOUNDS.
#include "mesh_internal.cuh"

#include <algorithm>

namespace mesh {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int WT = 256;           // threads per CTA
constexpr int WPT = 16;           // vertices per thread
constexpr int WB = WT * WPT;      // vertices per block
constexpr long long OWN = (long long)(1ull << 63);

__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdull;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ull;
    x ^= x >> 33;
    return x;
}

// Exclusive scan of one value per thread across the CTA; returns the prefix,
// *total the CTA's sum.
__device__ __forceinline__ long long cta_scan(long long v, long long *s_w, long long *total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    long long inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long u = __shfl_up_sync(FULL, inc, o);
        if (lane >= o) inc += u;
    }
    if (lane == 31) s_w[w] = inc;
    __syncthreads();
    if (w == 0) {
        const long long x = lane < nw ? s_w[lane] : 0;
        long long xi = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long u = __shfl_up_sync(FULL, xi, o);
            if (lane >= o) xi += u;
        }
        if (lane < nw) s_w[lane] = xi - x;
        if (lane == 31) s_w[32] = xi;
    }
    __syncthreads();
    const long long r = s_w[w] + inc - v;
    *total = s_w[32];
    __syncthreads();
    return r;
}

// dev_nv (batches): the vertex count, read on the device, at most nv
__global__ void __launch_bounds__(WT) k_weld_count(const long long *vkey, int64_t nv, long long *bsum,
                                                   const int64_t *dev_nv = nullptr) {
    __shared__ long long s_w[33];
    if (dev_nv) nv = min(nv, dev_nv[0]);
    const int64_t v0 = (int64_t)blockIdx.x * WB + (int64_t)threadIdx.x * WPT;
    long long c = 0;
#pragma unroll
    for (int k = 0; k < WPT; k++)
        if (v0 + k < nv) c += vkey[v0 + k] < 0;  // bit 63: owned
    long long tot;
    cta_scan(c, s_w, &tot);
    if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

// In place: bsum[b] becomes the welded id of block b's first owned vertex;
// bsum[nb] the number of welded vertices.
__global__ void __launch_bounds__(1024) k_weld_scan(long long *bsum, int64_t nb) {
    __shared__ long long s_w[33];
    const int64_t per = (nb + blockDim.x - 1) / blockDim.x;
    const int64_t b0 = min(nb, (int64_t)threadIdx.x * per), b1 = min(nb, b0 + per);
    long long s = 0;
    for (int64_t b = b0; b < b1; b++) s += bsum[b];
    long long tot;
    long long run = cta_scan(s, s_w, &tot);
    for (int64_t b = b0; b < b1; b++) {
        const long long v = bsum[b];
        bsum[b] = run;
        run += v;
    }
    if (threadIdx.x == 0) bsum[nb] = tot;
}

template <class F>
__global__ void __launch_bounds__(WT) k_weld_place(const long long *vkey, int64_t nv, const long long *bsum,
                                                   const F *verts, F *wverts, unsigned long long *hkey,
                                                   long long *hval, int64_t hcap, unsigned *err,
                                                   const int64_t *dev_nv = nullptr) {
    __shared__ long long s_w[33];
    if (dev_nv) nv = min(nv, dev_nv[0]);
    const int64_t v0 = (int64_t)blockIdx.x * WB + (int64_t)threadIdx.x * WPT;
    long long c = 0;
#pragma unroll
    for (int k = 0; k < WPT; k++)
        if (v0 + k < nv) c += vkey[v0 + k] < 0;
    long long tot;
    long long id = bsum[blockIdx.x] + cta_scan(c, s_w, &tot);
    const unsigned long long mask = (unsigned long long)hcap - 1;
    for (int k = 0; k < WPT; k++) {
        const int64_t j = v0 + k;
        if (j >= nv || vkey[j] >= 0) continue;
        wverts[3 * id] = verts[3 * j];
        wverts[3 * id + 1] = verts[3 * j + 1];
        wverts[3 * id + 2] = verts[3 * j + 2];
        const unsigned long long key = (unsigned long long)(vkey[j] & ~OWN) + 1;  // 0 marks an empty slot
        unsigned long long h = mix64(key) & mask;
        int64_t probe = 0;
        for (; probe < hcap; probe++, h = (h + 1) & mask) {
            const unsigned long long prev = atomicCAS(hkey + h, 0ull, key);
            if (prev == 0ull) {
                hval[h] = id;
                break;
            }
            if (prev == key) {  // two owners of one edge: not a welded mesh
                atomicOr(err, ERR_BOUNDS);
                break;
            }
        }
        if (probe == hcap) atomicOr(err, ERR_BOUNDS);
        id++;
    }
}

__global__ void __launch_bounds__(WT) k_weld_faces(const long long *vkey, int64_t nv, int64_t *faces, int64_t n,
                                                   const unsigned long long *hkey, const long long *hval,
                                                   int64_t hcap, unsigned *err) {
    const unsigned long long mask = (unsigned long long)hcap - 1;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = faces[i] - 1;
        if (j < 0 || j >= nv) {
            atomicOr(err, ERR_BOUNDS);
            continue;
        }
        const unsigned long long key = (unsigned long long)(vkey[j] & ~OWN) + 1;
        unsigned long long h = mix64(key) & mask;
        long long id = -1;
        for (int64_t probe = 0; probe < hcap; probe++, h = (h + 1) & mask) {
            const unsigned long long k = hkey[h];
            if (k == key) {
                id = hval[h];
                break;
            }
            if (k == 0ull) break;
        }
        if (id < 0) {
            atomicOr(err, ERR_BOUNDS);
            continue;
        }
        faces[i] = id + 1;
    }
}

// Batches: the welded first vertex of every volume v (row n: the welded total)
// is the number of owned vertices before its first ordinary vertex -- the
// scanned count of its block plus the owned vertices of that block before it
// (a warp per volume); the face rows are unchanged.
__global__ void __launch_bounds__(256) k_weld_vol_offsets(const long long *vkey, int64_t nvmax, const int64_t *tot,
                                                          const long long *bsum, const int64_t *vol_off, int n,
                                                          int64_t *woff) {
    const int lane = threadIdx.x & 31;
    const int64_t v = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (v > n) return;  // warp-uniform
    const int64_t nv = min(nvmax, tot[0]);
    const int64_t i = min(nv, vol_off[2 * v]);
    const int64_t b0 = (i / WB) * WB;
    long long c = 0;
    for (int64_t j = b0 + lane; j < i; j += 32) c += vkey[j] < 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(FULL, c, o);
    if (lane == 0) {
        woff[2 * v] = bsum[i / WB] + c;
        woff[2 * v + 1] = vol_off[2 * v + 1];
    }
}

// Batches: every face vertex (1-based within its volume) becomes the welded
// vertex of its edge, 1-based within the volume's welded vertices.  A face's
// volume is the last one whose first face is at or before it (volumes without
// faces share their successor's first face).
__global__ void __launch_bounds__(WT) k_weld_faces_batch(const long long *vkey, int64_t nvmax, int64_t nfmax,
                                                         const int64_t *tot, int64_t *faces, const int64_t *vol_off,
                                                         const int64_t *woff, int n,
                                                         const unsigned long long *hkey, const long long *hval,
                                                         int64_t hcap, unsigned *err) {
    const int64_t nv = min(nvmax, tot[0]), m = 3 * min(nfmax, tot[1]);
    const unsigned long long mask = (unsigned long long)hcap - 1;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t f = i / 3;
        int lo = 0, hi = n - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (vol_off[2 * mid + 1] <= f) lo = mid;
            else hi = mid - 1;
        }
        const int64_t j = vol_off[2 * lo] + faces[i] - 1;
        if (j < 0 || j >= nv) {
            atomicOr(err, ERR_BOUNDS);
            continue;
        }
        const unsigned long long key = (unsigned long long)(vkey[j] & ~OWN) + 1;
        unsigned long long h = mix64(key) & mask;
        long long id = -1;
        for (int64_t probe = 0; probe < hcap; probe++, h = (h + 1) & mask) {
            const unsigned long long k = hkey[h];
            if (k == key) {
                id = hval[h];
                break;
            }
            if (k == 0ull) break;
        }
        if (id < 0) {
            atomicOr(err, ERR_BOUNDS);
            continue;
        }
        faces[i] = id - woff[2 * lo] + 1;
    }
}

}  // namespace

// Hash slots for nv ordinary vertices (a power of two, at least twice the
// welded vertices, which are at most nv).
int64_t weld_hash_slots(int64_t nv) {
    int64_t h = 64;
    while (h < 2 * nv) h <<= 1;
    return h;
}
int64_t weld_blocks(int64_t nv) { return (nv + WB - 1) / WB; }

// Scratch: bsum [nb + 1], hkey [hcap], hval [hcap]; wverts nv * 3 elements.
cudaError_t launch_weld(const long long *vkey, int64_t nv, const void *verts, int out64, int64_t *faces, int64_t nf,
                        long long *bsum, void *wverts, unsigned long long *hkey, long long *hval, int64_t hcap,
                        unsigned *err, int sms, cudaStream_t s) {
    const int64_t nb = weld_blocks(nv);
    cudaError_t e = cudaMemsetAsync(hkey, 0, (size_t)hcap * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    if (nb == 0) return cudaMemsetAsync(bsum, 0, sizeof(long long), s);
    k_weld_count<<<(unsigned)nb, WT, 0, s>>>(vkey, nv, bsum);
    k_weld_scan<<<1, 1024, 0, s>>>(bsum, nb);
    if (out64)
        k_weld_place<double><<<(unsigned)nb, WT, 0, s>>>(vkey, nv, bsum, (const double *)verts, (double *)wverts,
                                                         hkey, hval, hcap, err);
    else
        k_weld_place<float><<<(unsigned)nb, WT, 0, s>>>(vkey, nv, bsum, (const float *)verts, (float *)wverts,
                                                        hkey, hval, hcap, err);
    const int64_t n = 3 * nf;
    if (n > 0)
        k_weld_faces<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>((n + WT - 1) / WT, (int64_t)sms * 16)), WT,
                       0, s>>>(vkey, nv, faces, n, hkey, hval, hcap, err);
    return cudaGetLastError();
}

cudaError_t launch_weld_batch(const long long *vkey, int64_t nvmax, int64_t nfmax, const int64_t *tot,
                              const void *verts, int out64, int64_t *faces, const int64_t *vol_off, int n,
                              int64_t *woff, long long *bsum, void *wverts, unsigned long long *hkey, long long *hval,
                              int64_t hcap, unsigned *err, int sms, cudaStream_t s) {
    const int64_t nb = weld_blocks(nvmax);
    cudaError_t e = cudaMemsetAsync(hkey, 0, (size_t)hcap * sizeof(unsigned long long), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(bsum, 0, (size_t)(nb + 1) * sizeof(long long), s);
    if (e != cudaSuccess) return e;
    if (nb > 0) {
        k_weld_count<<<(unsigned)nb, WT, 0, s>>>(vkey, nvmax, bsum, tot);
        k_weld_scan<<<1, 1024, 0, s>>>(bsum, nb);
        if (out64)
            k_weld_place<double><<<(unsigned)nb, WT, 0, s>>>(vkey, nvmax, bsum, (const double *)verts,
                                                             (double *)wverts, hkey, hval, hcap, err, tot);
        else
            k_weld_place<float><<<(unsigned)nb, WT, 0, s>>>(vkey, nvmax, bsum, (const float *)verts,
                                                            (float *)wverts, hkey, hval, hcap, err, tot);
    }
    k_weld_vol_offsets<<<(unsigned)((32 * ((int64_t)n + 1) + 255) / 256), 256, 0, s>>>(vkey, nvmax, tot, bsum, vol_off,
                                                                                      n, woff);
    const int64_t m = 3 * nfmax;
    if (m > 0 && n > 0)
        k_weld_faces_batch<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>((m + WT - 1) / WT, (int64_t)sms * 16)),
                             WT, 0, s>>>(vkey, nvmax, nfmax, tot, faces, vol_off, woff, n, hkey, hval, hcap, err);
    return cudaGetLastError();
}

}  // namespace mesh
