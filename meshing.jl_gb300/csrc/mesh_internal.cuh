// Internal definitions shared by the host runtime (mesh_api.cu) and the
// kernels (k_*.cu).  Not part of the public ABI.
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "meshing_gb300.h"  // include/ (on the include path)

namespace mesh {

// Tiling.  A warp tile covers 32 consecutive x samples (one per lane) and
// WY+1 consecutive y sample rows, and walks z.  Lane 31 only supplies the
// x+1 sample of lane 30, so a tile holds 31 cells in x (30 for the emit
// kernels that also need the -x neighbour cell, kept in lane 0).
constexpr int WY = 4;            // cell rows per warp tile
constexpr int WARPS = 8;         // warps per CTA
constexpr int TILE_X = 31;       // cells per tile in x (classify, MC emit)
constexpr int TILE_XH = 30;      // cells per tile in x (MT / NSN emit, with -x halo)
constexpr int ZC = 8;            // cells per activity chunk in z
constexpr int NCNT = 3;          // per-piece counters: vertices, faces, active cells
constexpr int ENT_BLOCK = 256;   // active-cell entries per expansion block
constexpr int POS_BITS = 21;     // bits per coordinate in a packed cell position

// Error bits of the device error word.
constexpr unsigned ERR_SCAN_TIMEOUT = 1u;
constexpr unsigned ERR_CAPACITY = 2u;
constexpr unsigned ERR_BOUNDS = 4u;
constexpr unsigned ERR_STAGE = 16u;  // the staged entry list was too short (8 is the TMA wait)

struct BatchVol;

struct Plan {
    // volume (Julia layout: x fastest)
    const void *vol;
    int64_t nx, ny, nz;
    int32_t cx, cy, cz;  // cells = samples - 1
    int32_t T, alg;
    int32_t out64;       // output eltype is Float64
    // classification thresholds: v < iso  <=>  v < thr (exact, in the data type)
    float thr_f;
    double thr_d;
    int32_t thr_i;       // UInt16 data
    int64_t thr_l;       // Int32 / Int64 data: v < iso  <=>  v < thr_l, or every v (thr_all)
    int32_t thr_all;
    // Int64 iso on Int64 data: (iso - v1) is an Int64 difference (wrapping)
    int64_t iso_l;
    int32_t iso_int;
    // iso as it enters (iso - v1)/(v2 - v1)
    float isoq_f;
    double isoq_d;
    // MT clamp bounds eps and one(T)-eps, in the clamp type
    float eps_f, hi_f;
    double eps_d, hi_d;
    uint32_t own[8];     // MT: edges owned by a cell, by (x==0)|(y==0)<<1|(z==0)<<2
    // LinRange node coordinates: exact values (L may be Float32) stored as double,
    // the same rounded to float, and the node spacings L(p[i+1]-p[i]).
    const double *xp, *yp, *zp;
    const double *dx, *dy, *dz;
    const float *xpf, *ypf, *zpf;
    const float *dxf, *dyf, *dzf;
    // float pairs hi + lo of the node coordinates and spacings (for the exact
    // float fast path of Float64 positions rounded to Float32): split[k][ntab]
    // with k = 0 p_hi, 1 p_lo, 2 d_hi, 3 d_lo, nodes of x, then y, then z
    const float *split;
    int64_t ntab;
    int32_t force_fp64;   // disable the float fast path (diagnostics)
    // z segments and activity chunks
    int32_t zs, nseg, chunks_per_seg, nchunks;
    int32_t tiles_x, tiles_y;  // classify tiling (TILE_X x WY cells)
    // scratch
    int64_t pstride;      // elements between the counters' arrays in cnt / base
    uint32_t *cnt;        // [NCNT][nseg][cy][cx] per-piece vertex / face / active-cell counts
    int64_t *base;        // [NCNT][nseg][cy][cx] exclusive prefix in traversal order
    uint8_t *flags;       // [nchunks][tiles_x][cy] 1 if the tile row has an active cell
    // Marching Cubes, single volume (null otherwise): [tiles_x][cy][nchunks] bit l
    // set when cell column tx * TILE_X + l of that row has an active cell in the chunk
    uint32_t *cmask;
    unsigned long long *scan_state;  // [NCNT][scan tiles] decoupled look-back words
    unsigned int *scan_ticket;
    int64_t *totals;      // [NCNT] total vertices, faces, active cells
    unsigned int *err;    // device error word
    unsigned int *work;   // work-item counter of the persistent kernels
    // welded Marching Cubes: per emitted vertex, its lattice edge
    // (axis + 3 * linear index of the edge's lower node), bit 63 set when the
    // emitting cell is the edge's first cell in emission order (null: not written)
    long long *vkey;
    // list of active cells (Marching Cubes): packed x | y << 21 | z << 42,
    // case, the 8 corner values; in emission order with, for every 256th
    // entry, the vertex / face offsets of that entry (ent_side), or in the
    // order the walk found them with each entry's vertex / face rank inside
    // its piece (ent_rank) and *stage_next slots handed out
    unsigned long long *ent_pos;
    uint8_t *ent_cs;
    void *ent_val;
    long long *ent_side;
    uint2 *ent_rank;
    unsigned long long *stage_next;
    int64_t ent_cap;
    // outputs
    void *verts;
    int64_t *faces;
    int64_t verts_cap, faces_cap;
    int32_t scan_spin_limit;
    // batches (Marching Cubes over many volumes in one pass): per-volume
    // descriptors, the volume of each work item and of each scan tile, the
    // volume of each active-cell entry, and the first vertex / face of every
    // volume ([nvols + 1][2], the last row the totals)
    const BatchVol *bvols;
    const uint32_t *item_vol, *stile_vol;
    uint32_t *ent_vol;
    int64_t *vol_off;
    int64_t nitems;
    int32_t nvols, nstiles;
    int32_t vol_outputs;  // 1: every volume writes to its own BatchVol::verts / faces
    // x window (mesh_set_x_window): global x of the volume's sample 0, for the
    // grid-boundary rules of MT / NSN; with xhalo, the volume's first cell column
    // is the previous slab's last one -- counted (its vertices come first in the
    // scan) but not emitted, and every emitted vertex, face and face index is
    // shifted down by that column's totals (base of piece (seg 0, y 0, x 1))
    int64_t xg0;
    int32_t xhalo;
    // sub-range launches of the pipelined host path (zero: the whole volume):
    // classify z segments seg0 .. seg1 - 1; compact the x tiles tx0 .. tx0 + ntx - 1;
    // expand list entries e_lo .. e_hi - 1
    int32_t seg0, seg1, tx0, ntx;
    int64_t e_lo, e_hi;
};

// One volume of a batch.  Its work items, pieces, activity bytes and scan
// tiles are ranges of the batch's arrays starting at item0, piece0, flag0 and
// stile0; its coordinate tables are a block at `tabs` (k_tables.cu layout).
// With Plan::vol_outputs its mesh goes to its own verts / faces (room for
// vcap / fcap) instead of the batch's concatenated outputs.
struct BatchVol {
    const void *vol;
    const double *tabs;
    int64_t nx, ny, nz;
    int32_t cx, cy, cz, tiles_x, tiles_y, nseg, zs, chunks_per_seg, nchunks, stile0;
    int64_t item0, piece0, flag0;
    void *verts;
    int64_t *faces;
    int64_t vcap, fcap;
    int64_t kbase;  // welded batches: the volume's lattice-edge keys start here
};

// Bytes per sample of a volume dtype.
inline __host__ __device__ size_t dtype_size(int T) {
    return (T == MESH_DT_I8 || T == MESH_DT_U8) ? 1
           : (T == MESH_DT_U16 || T == MESH_DT_F16 || T == MESH_DT_I16) ? 2
           : (T == MESH_DT_F32 || T == MESH_DT_I32) ? 4 : 8;
}

inline __host__ __device__ int64_t npieces(const Plan &p) { return (int64_t)p.nseg * p.cy * p.cx; }

// Coordinate tables of one volume (pointers into its table block).
struct Tabs {
    const double *xp, *yp, *zp, *dx, *dy, *dz;
    const float *xpf, *ypf, *zpf, *dxf, *dyf, *dzf, *split;
    int64_t ntab, nx, ny;
};
inline __host__ __device__ Tabs tabs_of(const Plan &p) {
    return Tabs{p.xp, p.yp, p.zp, p.dx, p.dy, p.dz, p.xpf, p.ypf, p.zpf, p.dxf, p.dyf, p.dzf, p.split,
                p.ntab, p.nx, p.ny};
}
// The tables of a block at dp (k_tables.cu layout) for nx, ny, nz nodes.
inline __host__ __device__ Tabs tabs_at(const double *dp, int64_t nx, int64_t ny, int64_t nz) {
    const int64_t ntab = nx + ny + nz;
    const double *dd = dp + ntab;
    const float *fp = (const float *)(dp + 2 * ntab), *fd = fp + ntab;
    return Tabs{dp, dp + nx, dp + nx + ny, dd, dd + nx, dd + nx + ny, fp, fp + nx, fp + nx + ny,
                fd, fd + nx, fd + nx + ny, fp + 2 * ntab, ntab, nx, ny};
}
inline __host__ __device__ void set_tabs(Plan &P, const Tabs &t) {
    P.xp = t.xp; P.yp = t.yp; P.zp = t.zp; P.dx = t.dx; P.dy = t.dy; P.dz = t.dz;
    P.xpf = t.xpf; P.ypf = t.ypf; P.zpf = t.zpf; P.dxf = t.dxf; P.dyf = t.dyf; P.dzf = t.dzf;
    P.split = t.split;
    P.ntab = t.ntab;
}
// The batch plan p seen as a plan of its volume b alone (shared arrays offset).
inline __host__ __device__ Plan vol_view(const Plan &p, const BatchVol &b) {
    Plan v = p;
    v.vol = b.vol;
    v.nx = b.nx; v.ny = b.ny; v.nz = b.nz;
    v.cx = b.cx; v.cy = b.cy; v.cz = b.cz;
    v.tiles_x = b.tiles_x; v.tiles_y = b.tiles_y;
    v.nseg = b.nseg; v.zs = b.zs; v.chunks_per_seg = b.chunks_per_seg; v.nchunks = b.nchunks;
    v.cnt = p.cnt + b.piece0;
    v.base = p.base + b.piece0;
    v.flags = p.flags + b.flag0;
    set_tabs(v, tabs_at(b.tabs, b.nx, b.ny, b.nz));
    return v;
}
inline __host__ __device__ int64_t piece(const Plan &p, int seg, int y, int x) {
    return ((int64_t)seg * p.cy + y) * p.cx + x;
}

// Coordinate tables (k_tables.cu): bytes for ntab = nx+ny+nz nodes, and the
// Plan's pointers into a table block at dp.
inline size_t table_bytes(int64_t ntab) {
    return (size_t)ntab * 2 * (sizeof(double) + sizeof(float)) + (size_t)ntab * 4 * sizeof(float);
}
inline void bind_tables(Plan &P, const double *dp, int64_t nx, int64_t ny, int64_t nz) {
    set_tabs(P, tabs_at(dp, nx, ny, nz));
}

// Welded Marching Cubes (k_weld.cu): blocks of the ownership scan and hash slots
// for nv per-cell vertices; launch_weld welds verts / faces (faces in place) into
// wverts, bsum[nb] = the welded vertex count.
int64_t weld_blocks(int64_t nv);
int64_t weld_hash_slots(int64_t nv);
cudaError_t launch_weld(const long long *vkey, int64_t nv, const void *verts, int out64, int64_t *faces, int64_t nf,
                        long long *bsum, void *wverts, unsigned long long *hkey, long long *hval, int64_t hcap,
                        unsigned *err, int sms, cudaStream_t s);
// The same over a batch: the counts are read on the device (tot[0] vertices,
// tot[1] faces, at most nvmax / nfmax), faces are 1-based within their volume
// (first vertex / face of volume v at vol_off[2v], vol_off[2v + 1]; row n the
// totals) before and after, and woff receives the welded rows.
cudaError_t launch_weld_batch(const long long *vkey, int64_t nvmax, int64_t nfmax, const int64_t *tot,
                              const void *verts, int out64, int64_t *faces, const int64_t *vol_off, int n,
                              int64_t *woff, long long *bsum, void *wverts, unsigned long long *hkey, long long *hval,
                              int64_t hcap, unsigned *err, int sms, cudaStream_t s);

// Launchers (each returns cudaError_t of the launch).
// xoff / nxt: the volume is x nodes xoff .. xoff+nx-1 of an axis of nxt nodes (0, 0: the whole axis).
cudaError_t launch_tables(double *tabs, int64_t nx, int64_t ny, int64_t nz, const double *range, int L32,
                          cudaStream_t s, int64_t xoff = 0, int64_t nxt = 0);
// Tables of many volumes: job i fills the block at dst[i] (one CTA row per job).
struct TabJob {
    double *dst;
    int64_t nx, ny, nz;
    double range[6];
};
cudaError_t launch_tables_batch(const TabJob *jobs, int njobs, int64_t max_ntab, int L32, cudaStream_t s);
// Batched Marching Cubes stages (k_classify.cu, k_scan.cu, k_emit_mc.cu);
// ctas: CTAs per SM of the persistent kernels (0 = as many as fit), threads:
// threads per scan CTA.
cudaError_t launch_classify_batch(const Plan &p, int ctas, cudaStream_t s);
// per_volume: every volume is at most a few 32-column groups wide -- chain the
// volumes, one CTA each (scan state for NCNT x nvols entries)
cudaError_t launch_scan_batch(const Plan &p, int threads, cudaStream_t s, bool per_volume = false);
cudaError_t launch_compact_batch(const Plan &p, int ctas, cudaStream_t s);
cudaError_t launch_expand_batch(const Plan &p, int Q64, int P64, cudaStream_t s);
cudaError_t launch_classify(const Plan &p, cudaStream_t s, int seg0 = 0, int nsegs = 0);  // nsegs 0: all
// A few values of a device int64 array for the host: dst[i] = src[idx[i]], i < n.
constexpr int GATHER_MAX = 32;
struct GatherIdx {
    int64_t idx[GATHER_MAX];
    int n;
};
cudaError_t launch_gather(const int64_t *src, const GatherIdx &g, int64_t *dst, cudaStream_t s);
cudaError_t launch_scan(const Plan &p, cudaStream_t s);
cudaError_t launch_emit(const Plan &p, int Q64, int A64, int P64, cudaStream_t s);
// Marching Cubes emitted straight from the volume (k_direct_mc.cu): needs cmask.
cudaError_t launch_direct_mc(const Plan &p, int Q64, int P64, cudaStream_t s);
// Marching Cubes in one walk: classify + stage entries, then expand them.
constexpr int STG_BLK = 128;  // staging slots a walking warp takes at a time
cudaError_t launch_walk_mc(const Plan &p, cudaStream_t s);
cudaError_t launch_expand_staged_mc(const Plan &p, int Q64, int P64, cudaStream_t s);

}  // namespace mesh

#ifdef __CUDACC__
namespace mesh {

// Round-to-nearest arithmetic that the compiler may not contract into FMA,
// matching Julia's separately rounded `+ - * /`.
template <class F> struct Ar;
template <> struct Ar<float> {
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
};
template <> struct Ar<double> {
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
    static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
    static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
    static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
};

// A Float16 sample, kept as its IEEE binary16 bits.  Every Float16 value is a
// Float32 value, so it converts exactly; T(0) is the zero sample.
struct h16 {
    uint16_t b;
    h16() = default;
    __host__ __device__ constexpr explicit h16(int) : b(0) {}
    __device__ __forceinline__ operator float() const { return __half2float(__ushort_as_half(b)); }
};
static_assert(sizeof(h16) == 2, "binary16 storage");

// v < iso, exact, in the data type.
__device__ __forceinline__ bool below(h16 v, const Plan &p) { return (float)v < p.thr_f; }
__device__ __forceinline__ bool below(float v, const Plan &p) { return v < p.thr_f; }
__device__ __forceinline__ bool below(double v, const Plan &p) { return v < p.thr_d; }
__device__ __forceinline__ bool below(uint16_t v, const Plan &p) { return (int32_t)v < p.thr_i; }
__device__ __forceinline__ bool below(uint8_t v, const Plan &p) { return (int32_t)v < p.thr_i; }
__device__ __forceinline__ bool below(int8_t v, const Plan &p) { return (int64_t)v < p.thr_l || p.thr_all; }
__device__ __forceinline__ bool below(int16_t v, const Plan &p) { return (int64_t)v < p.thr_l || p.thr_all; }
__device__ __forceinline__ bool below(int32_t v, const Plan &p) { return (int64_t)v < p.thr_l || p.thr_all; }
__device__ __forceinline__ bool below(int64_t v, const Plan &p) { return v < p.thr_l || p.thr_all; }

// A Float32 value widened to Q.  To Float64 the widening of a normal or zero
// value only moves bits (exponent rebiased by 1023 - 127, significand shifted
// up by 29), done here on the integer pipes; subnormals, Inf and NaN take the
// conversion instruction.
template <class Q> __device__ __forceinline__ Q widen(float v) { return (Q)v; }
template <> __device__ __forceinline__ double widen<double>(float v) {
    const uint32_t u = __float_as_uint(v), e = (u >> 23) & 0xffu;
    const unsigned long long sgn = (unsigned long long)(u & 0x80000000u) << 32;
    if (e != 0u && e != 0xffu)
        return __longlong_as_double((long long)(sgn | ((unsigned long long)(e + 896u) << 52) |
                                                ((unsigned long long)(u & 0x7fffffu) << 29)));
    if ((u << 1) == 0u) return __longlong_as_double((long long)sgn);
    return (double)v;
}

// v2 - v1 in the data type (UInt16 wraps), then converted to Q.
template <class Q> __device__ __forceinline__ Q tdiff(float v2, float v1) { return widen<Q>(__fsub_rn(v2, v1)); }
// Float16 - Float16 is a Float16: the Float32 difference of two Float16 values
// is exact, so rounding it to Float16 once gives the IEEE half subtraction.
template <class Q> __device__ __forceinline__ Q tdiff(h16 v2, h16 v1) {
    return (Q)__half2float(__float2half_rn(__fsub_rn((float)v2, (float)v1)));
}
template <class Q> __device__ __forceinline__ Q tdiff(double v2, double v1) { return (Q)__dsub_rn(v2, v1); }
template <class Q> __device__ __forceinline__ Q tdiff(uint16_t v2, uint16_t v1) { return (Q)(uint16_t)(v2 - v1); }
template <class Q> __device__ __forceinline__ Q tdiff(uint8_t v2, uint8_t v1) { return (Q)(uint8_t)(v2 - v1); }
template <class Q> __device__ __forceinline__ Q tdiff(int8_t v2, int8_t v1) {
    return (Q)(int8_t)(uint8_t)((uint8_t)v2 - (uint8_t)v1);
}
template <class Q> __device__ __forceinline__ Q tdiff(int16_t v2, int16_t v1) {
    return (Q)(int16_t)(uint16_t)((uint16_t)v2 - (uint16_t)v1);
}
// machine-integer differences wrap; the conversion to Q rounds to nearest
template <class Q> __device__ __forceinline__ Q tdiff(int32_t v2, int32_t v1) {
    return (Q)(int32_t)((uint32_t)v2 - (uint32_t)v1);
}
template <class Q> __device__ __forceinline__ Q tdiff(int64_t v2, int64_t v1) {
    return (Q)(int64_t)((unsigned long long)v2 - (unsigned long long)v1);
}

template <class Q> __device__ __forceinline__ Q isoq(const Plan &p);
template <> __device__ __forceinline__ float isoq<float>(const Plan &p) { return p.isoq_f; }
template <> __device__ __forceinline__ double isoq<double>(const Plan &p) { return p.isoq_d; }

// (iso - v1) / (v2 - v1) in Julia's promoted types.
template <class Q, class T> __device__ __forceinline__ Q quotient(T v1, T v2, const Plan &p) {
    Q den = tdiff<Q>(v2, v1);
    Q num;
    if (std::is_integral<T>::value && sizeof(T) == 8 && p.iso_int)  // Int64 data, Int64 iso: Int64 (iso - v1)
        num = (Q)(int64_t)((unsigned long long)p.iso_l - (unsigned long long)(int64_t)v1);
    else if (std::is_same<T, float>::value)
        num = Ar<Q>::sub(isoq<Q>(p), widen<Q>((float)v1));
    else
        num = Ar<Q>::sub(isoq<Q>(p), (Q)v1);
    return Ar<Q>::div(num, den);
}

// Classification of IEEE values by their bits, so that Float64 tests stay off
// the (1/64-rate) FP64 pipe.
__device__ __forceinline__ bool bits_nan(float v) { return (__float_as_uint(v) << 1) > 0xff000000u; }
__device__ __forceinline__ bool bits_nan(double v) {
    return ((unsigned long long)__double_as_longlong(v) << 1) > 0xffe0000000000000ull;
}
__device__ __forceinline__ bool bits_finite(float v) { return (__float_as_uint(v) << 1) < 0xff000000u; }
__device__ __forceinline__ bool bits_finite(double v) {
    return ((unsigned long long)__double_as_longlong(v) << 1) < 0xffe0000000000000ull;
}
__device__ __forceinline__ bool bits_zero(float v) { return (__float_as_uint(v) << 1) == 0u; }
__device__ __forceinline__ bool bits_zero(double v) { return ((unsigned long long)__double_as_longlong(v) << 1) == 0ull; }

// Base.max / Base.min on IEEE floats: NaN propagates, -0.0 < +0.0.
template <class A> __device__ __forceinline__ A jl_max(A x, A y) {
    A d = Ar<A>::sub(x, y);
    if (bits_nan(x) || bits_nan(y)) return d;
    return signbit(d) ? y : x;
}
template <class A> __device__ __forceinline__ A jl_min(A x, A y) {
    A d = Ar<A>::sub(x, y);
    if (bits_nan(x) || bits_nan(y)) return d;
    return signbit(d) ? x : y;
}

// fl32(fl64(p1 + fl64(mu * d))) for a Float32 mu and Float64 p1, d given as
// float pairs (p1 = p1h + p1l, d = dh + dl up to 2^-48 relative), without FP64
// instructions.  A float-float estimate r of p1 + mu*d is formed with
// TwoProduct / TwoSum; together with the two Float64 roundings of the
// reference it lies within E = 2^-42 (|p1| + |mu d|) of the exact value (the
// analysis gives about 2^-44).  If no Float32 rounding boundary lies within E
// of r, the reference result rounds to the same float f = fl32(r) and the
// function returns true; otherwise (or near underflow/overflow) it returns
// false and the caller evaluates the Float64 expression.
__device__ __forceinline__ bool fast_f32_pos(float mu, float p1h, float p1l, float dh, float dl, float &out) {
    const float ph = __fmul_rn(mu, dh);
    const float pe = __fmaf_rn(mu, dh, -ph);  // exact: mu*dh == ph + pe
    const float ql = __fmul_rn(mu, dl);
    const float sh = __fadd_rn(p1h, ph);      // TwoSum(p1h, ph) = sh + se
    const float bb = __fsub_rn(sh, p1h);
    const float se = __fadd_rn(__fsub_rn(p1h, __fsub_rn(sh, bb)), __fsub_rn(ph, bb));
    const float lo = __fadd_rn(se, __fadd_rn(p1l, __fadd_rn(pe, ql)));
    const float f = __fadd_rn(sh, lo);
    const float t = __fadd_rn(__fsub_rn(sh, f), lo);  // r - f
    const unsigned fb = __float_as_uint(f) & 0x7fffffffu;
    const int e = (int)(fb >> 23);
    out = f;
    if (e < 64 || e > 190) return false;
    float hu = __uint_as_float((unsigned)(e - 24) << 23);  // half ulp of |f|
    if ((fb & 0x7fffffu) == 0u) hu = __fmul_rn(hu, 0.5f);  // power of two: the gap towards zero is half
    const float E = __fmul_rn(__fadd_rn(fabsf(p1h), fabsf(ph)), 0x1p-42f);
    return __fadd_rn(__fmul_rn(fabsf(t), 1.0000002f), E) < hu;
}

template <class T> __device__ __forceinline__ T shfl_down1(T v) { return __shfl_down_sync(0xffffffffu, v, 1); }
template <> __device__ __forceinline__ int8_t shfl_down1<int8_t>(int8_t v) {
    return (int8_t)__shfl_down_sync(0xffffffffu, (int)v, 1);
}
template <> __device__ __forceinline__ uint8_t shfl_down1<uint8_t>(uint8_t v) {
    return (uint8_t)__shfl_down_sync(0xffffffffu, (unsigned)v, 1);
}
template <> __device__ __forceinline__ int16_t shfl_down1<int16_t>(int16_t v) {
    return (int16_t)__shfl_down_sync(0xffffffffu, (int)v, 1);
}
template <> __device__ __forceinline__ h16 shfl_down1<h16>(h16 v) {
    h16 r;
    r.b = (uint16_t)__shfl_down_sync(0xffffffffu, (unsigned)v.b, 1);
    return r;
}
template <> __device__ __forceinline__ uint16_t shfl_down1<uint16_t>(uint16_t v) {
    return (uint16_t)__shfl_down_sync(0xffffffffu, (unsigned)v, 1);
}

template <class T> __device__ __forceinline__ T ldv(const T *p) { return __ldg(p); }
template <> __device__ __forceinline__ h16 ldv<h16>(const h16 *p) {
    h16 r;
    r.b = __ldg(reinterpret_cast<const unsigned short *>(p));
    return r;
}
template <> __device__ __forceinline__ uint16_t ldv<uint16_t>(const uint16_t *p) {
    return __ldg(reinterpret_cast<const unsigned short *>(p));
}

}  // namespace mesh
#endif
