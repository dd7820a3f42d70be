// Host runtime behind the C ABI (include/meshing_gb300.h).
//
// Turns a reference call isosurface(A, alg, X, Y, Z) into a launch plan:
// Julia's type promotion (src/marching_cubes.jl:31, src/marching_tetrahedra.jl:131)
// picks the arithmetic and output types, the LinRange node coordinates
// (src/marching_cubes.jl:36-38) are tabulated on the device with the exact
// Base.lerpi arithmetic (k_tables.cu), and the kernels run on the context's
// stream: classify -> scan -> emit.  Nothing waits on the host between
// launches.  Device scratch grows monotonically and is reused across calls.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "mesh_host.h"
#include "mesh_internal.cuh"
#include "mesh_tables.h"
#include "mesh_tma.cuh"

namespace mesh {
cudaError_t launch_classify_tma(const Plan &p, const CUtensorMap &map, cudaStream_t s);
cudaError_t launch_emit_mc(const Plan &p, int Q64, int P64, int stage, cudaStream_t s);
cudaError_t launch_emit_halo(const Plan &p, int Q64, int A64, int P64, cudaStream_t s);
size_t scan_scratch_bytes(const Plan &p);
}  // namespace mesh

using namespace mesh;

namespace mesh {

constexpr double EXACT_INT = 9007199254740992.0;  // 2^53

int fail(mesh_ctx *c, int status, const char *fmt, ...) {
    if (c) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        c->msg = buf;
    }
    return status;
}

int cuda_fail(mesh_ctx *c, cudaError_t e, const char *what) {
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return fail(c, MESH_ENOMEM, "%s: %s", what, cudaGetErrorString(e));
    }
    return fail(c, MESH_ECUDA, "%s: %s", what, cudaGetErrorString(e));
}

bool is_f32_exact(double v) { return std::isnan(v) || (double)(float)v == v; }

bool valid_scalar(int ty, double v) {
    switch (ty) {
    case MESH_DT_F64: return true;
    case MESH_DT_F32: return is_f32_exact(v);
    case MESH_DT_I64: return std::isfinite(v) && std::floor(v) == v && std::fabs(v) <= EXACT_INT;
    default: return false;
    }
}

// float(FT) is Float64 unless some participating type is Float32 and none is Float64.
int out_is_f64(const int *tys, int n) {
    int any32 = 0;
    for (int i = 0; i < n; i++) {
        if (tys[i] == MESH_DT_F64) return 1;
        if (tys[i] == MESH_DT_F32) any32 = 1;
    }
    return any32 ? 0 : 1;
}

int validate(mesh_ctx *c, int T, int64_t nx, int64_t ny, int64_t nz, const mesh_params *p) {
    if (!p) return fail(c, MESH_EINVAL, "params is NULL");
    if (T != MESH_DT_U16 && T != MESH_DT_F32 && T != MESH_DT_F64 && T != MESH_DT_I32 && T != MESH_DT_I64 &&
        T != MESH_DT_F16 && T != MESH_DT_I16 && T != MESH_DT_I8 && T != MESH_DT_U8)
        return fail(c, MESH_EINVAL, "unsupported volume dtype %d", T);
    // promote(Int, Float16) is Float16: (iso - v1) / (v2 - v1) would run in Float16 arithmetic
    if (T == MESH_DT_F16 && p && p->iso_type == MESH_DT_I64)
        return fail(c, MESH_EINVAL, "Float16 volumes take a Float32 or Float64 iso");
    if (p->alg != MESH_ALG_MC && p->alg != MESH_ALG_MT && p->alg != MESH_ALG_NSN && p->alg != MESH_ALG_MC_WELDED)
        return fail(c, MESH_EINVAL, "unknown algorithm %d", p->alg);
    if (p->iso_type != MESH_DT_F32 && p->iso_type != MESH_DT_F64 && p->iso_type != MESH_DT_I64)
        return fail(c, MESH_EINVAL, "unsupported iso type %d", p->iso_type);
    if (!valid_scalar(p->iso_type, p->iso)) return fail(c, MESH_EINVAL, "iso value not representable in its type");
    if (p->alg == MESH_ALG_MT) {
        if (p->eps_type != MESH_DT_F32 && p->eps_type != MESH_DT_F64)
            return fail(c, MESH_EINVAL, "unsupported eps type %d", p->eps_type);
        if (!valid_scalar(p->eps_type, p->eps)) return fail(c, MESH_EINVAL, "eps value not representable in its type");
    }
    if (p->range_type != MESH_DT_F32 && p->range_type != MESH_DT_F64 && p->range_type != MESH_DT_I64)
        return fail(c, MESH_EINVAL, "unsupported range type %d", p->range_type);
    for (int i = 0; i < 6; i++) {
        if (!std::isfinite(p->range[i])) return fail(c, MESH_EINVAL, "range endpoints must be finite");
        if (!valid_scalar(p->range_type, p->range[i])) return fail(c, MESH_EINVAL, "range endpoint not representable");
    }
    if (nx < 0 || ny < 0 || nz < 0) return fail(c, MESH_EINVAL, "negative dimension");
    const int64_t lim = (int64_t)1 << POS_BITS;
    if (nx > lim || ny > lim || nz > lim) return fail(c, MESH_ETOOLARGE, "dimension above 2^21");
    return MESH_OK;
}

void own_masks(uint32_t own[8]) {
    for (int bnd = 0; bnd < 8; bnd++) {
        uint32_t m = 0;
        for (int e = 0; e < 19; e++) {
            const int i1 = MT_EDGE_CORNERS[e][0], i2 = MT_EDGE_CORNERS[e][1];
            int za = 0;
            for (int k = 0; k < 3; k++)
                if (MT_CORNER_POS[i1][k] == 0 && MT_CORNER_POS[i2][k] == 0) za |= 1 << k;
            if ((za & ~bnd) == 0) m |= 1u << e;
        }
        own[bnd] = m;
    }
}

void set_types(Plan &P, int T, const mesh_params *p, int *Q64, int *A64, int *P64) {
    P.T = T;
    P.alg = p->alg;
    const int I = p->iso_type, E = p->eps_type, Rt = p->range_type;
    const int mt = p->alg == MESH_ALG_MT;
    // promote(typeof(iso), T); Int / Int divides in Float64
    *Q64 = T == MESH_DT_F64 || I == MESH_DT_F64 || (T != MESH_DT_F32 && I == MESH_DT_I64);
    const int L32 = Rt == MESH_DT_F32;
    *A64 = mt ? (*Q64 || E == MESH_DT_F64) : *Q64;
    *P64 = *A64 || !L32;
    if (!mt) *P64 = *Q64 || !L32;
    const int tys[4] = {Rt, T, I, E};
    P.out64 = out_is_f64(tys, mt ? 4 : 3);

    const double iso = p->iso;
    // thresholds: v < iso  <=>  v < thr in the data type
    {
        float f = (float)iso;
        if (!std::isnan(iso) && (double)f < iso) f = std::nextafter(f, INFINITY);
        P.thr_f = f;
        P.thr_d = iso;
        double ce = std::ceil(iso);
        if (std::isnan(iso)) ce = 0;
        P.thr_i = (int32_t)std::min(65536.0, std::max(0.0, ce));  // UInt16 / UInt8 data
        // Int8 / Int16 / Int32 / Int64 data: x < iso  <=>  x < ceil(iso), exact for every Int64 x
        P.thr_all = 0;
        if (std::isnan(iso)) {
            P.thr_l = INT64_MIN;                      // nothing is below NaN
        } else if (ce >= 9223372036854775808.0) {
            P.thr_l = INT64_MAX;
            P.thr_all = 1;                            // beyond every Int64
        } else if (ce < -9223372036854775808.0) {
            P.thr_l = INT64_MIN;
        } else {
            P.thr_l = (int64_t)ce;
        }
        P.iso_int = T == MESH_DT_I64 && I == MESH_DT_I64;
        P.iso_l = I == MESH_DT_I64 ? (int64_t)iso : 0;
    }
    P.isoq_d = iso;
    P.isoq_f = (float)iso;
    if (mt) {
        const int te64 = T == MESH_DT_F64 || E == MESH_DT_F64;  // promote(T, E)
        const double hi = te64 ? 1.0 - p->eps : (double)(1.0f - (float)p->eps);
        P.eps_d = p->eps;
        P.hi_d = hi;
        P.eps_f = (float)p->eps;
        P.hi_f = (float)hi;
        own_masks(P.own);
    }
}

}  // namespace mesh

namespace {

void count_kernels(mesh_ctx *c, int stage, int n);

// Copy stream, events and split-point buffers of the pipelined host path.
int ensure_pipe(mesh_ctx *c) {
    if (c->copy) return MESH_OK;
    cudaError_t e = cudaStreamCreateWithFlags(&c->copy, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_ready, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_done, cudaEventDisableTiming);
    for (int g = 0; g < PIPE_MAX && e == cudaSuccess; g++) e = cudaEventCreateWithFlags(&c->ev_part[g], cudaEventDisableTiming);
    if (e == cudaSuccess) e = c->gat.ensure(GATHER_MAX * sizeof(int64_t));
    if (e == cudaSuccess && !c->h_gat) e = cudaHostAlloc((void **)&c->h_gat, GATHER_MAX * sizeof(int64_t), cudaHostAllocDefault);
    if (e != cudaSuccess) {
        // leave no half-made pipeline behind: the next call retries from scratch
        for (cudaEvent_t &ev : c->ev_part)
            if (ev) cudaEventDestroy(ev), ev = nullptr;
        if (c->ev_ready) cudaEventDestroy(c->ev_ready), c->ev_ready = nullptr;
        if (c->ev_done) cudaEventDestroy(c->ev_done), c->ev_done = nullptr;
        if (c->copy) cudaStreamDestroy(c->copy);
        c->copy = nullptr;
        return cuda_fail(c, e, "pipeline stream");
    }
    return MESH_OK;
}

// Host volume upload in c->ngroups groups of z segments on the copy stream, each
// group classified on the compute stream as soon as it has arrived: group g holds
// the sample planes its segments read (segment s reads planes s*zs ..
// min((s+1)*zs, cz)).  Copies and launches are enqueued alternately, so that a
// pageable source (whose copies return only once staged) overlaps too.
cudaError_t upload_and_classify(mesh_ctx *c) {
    const Plan &P = c->plan;
    const size_t plane = (size_t)P.nx * P.ny * dtype_size(P.T);
    cudaError_t e = cudaEventRecord(c->ev_ready, c->stream);  // earlier work on the volume buffer
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->copy, c->ev_ready, 0);
    int64_t p0 = 0;
    int s0 = 0;
    for (int g = 0; g < c->ngroups && e == cudaSuccess; g++) {
        const int s1 = (int)((int64_t)(g + 1) * P.nseg / c->ngroups);
        const int64_t p1 = g + 1 == c->ngroups ? P.nz : std::min<int64_t>((int64_t)s1 * P.zs, P.nz - 1) + 1;
        if (p1 > p0)
            e = cudaMemcpyAsync((char *)c->vol.ptr + p0 * plane, (const char *)c->upl_src + p0 * plane,
                                (size_t)(p1 - p0) * plane, cudaMemcpyHostToDevice, c->copy);
        if (e == cudaSuccess) e = cudaEventRecord(c->ev_part[g], c->copy);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(c->stream, c->ev_part[g], 0);
        if (e == cudaSuccess && s1 > s0) e = launch_classify(P, c->stream, s0, s1 - s0);
        p0 = std::max(p0, p1);
        s0 = s1;
    }
    return e;
}

bool one_walk(const mesh_ctx *c);
bool direct_mc(const mesh_ctx *c);

int prepare(mesh_ctx *c, const void *vol, int T, int64_t nx, int64_t ny, int64_t nz, int vol_on_device,
            const mesh_params *p) {
    Plan &P = c->plan;
    P = Plan{};
    c->have_plan = 0;
    c->ngroups = 1;
    P.nx = nx; P.ny = ny; P.nz = nz;
    P.cx = (int32_t)(nx - 1); P.cy = (int32_t)(ny - 1); P.cz = (int32_t)(nz - 1);
    set_types(P, T, p, &c->Q64, &c->A64, &c->P64);
    const int L32 = p->range_type == MESH_DT_F32;
    // welded Marching Cubes runs the Marching Cubes kernels, then welds
    c->weld = p->alg == MESH_ALG_MC_WELDED;
    if (c->weld) P.alg = MESH_ALG_MC;
    // x window: MT / NSN take the grid-boundary rules at the whole volume's x = 0; with
    // a halo, the volume's first cell column is the previous slab's last (counted, not
    // emitted)
    P.xg0 = c->win_nx ? c->win_x0 : 0;
    P.xhalo = c->win_nx && c->win_halo;
    if (P.xhalo && P.alg != MESH_ALG_MT && P.alg != MESH_ALG_NSN)
        return fail(c, MESH_EINVAL, "a halo column is for MarchingTetrahedra / NaiveSurfaceNets slabs");

    // tiling
    P.tiles_x = (P.cx + TILE_X - 1) / TILE_X;
    P.tiles_y = (P.cy + WY - 1) / WY;
    const int64_t per_seg = (int64_t)P.tiles_x * P.tiles_y;
    const int64_t target = (int64_t)c->sms * 64;
    const int maxseg = (P.cz + ZC - 1) / ZC;
    int nseg = (int)std::min<int64_t>(maxseg, std::max<int64_t>(1, (target + per_seg - 1) / per_seg));
    // a host volume uploaded in groups of z segments (upload_and_classify) gets at
    // least PIPE_MAX segments, so that all but the last group's classification
    // runs under the upload (a mapped host volume read in place is not uploaded)
    const size_t vbytes0 = (size_t)nx * ny * nz * dtype_size(T);
    if (!vol_on_device && !c->zerocopy && c->pipe_bytes > 0 && (int64_t)vbytes0 >= c->pipe_bytes && c->tma_env != 1 &&
        !c->one_walk)
        nseg = std::min(maxseg, std::max(nseg, PIPE_MAX));
    int zs = (P.cz + nseg - 1) / nseg;
    zs = (zs + ZC - 1) / ZC * ZC;
    P.zs = zs;
    P.nseg = (P.cz + zs - 1) / zs;
    P.chunks_per_seg = zs / ZC;
    P.nchunks = P.nseg * P.chunks_per_seg;
    if ((P.tiles_y + WARPS - 1) / WARPS > 65535 || P.nseg > 65535)
        return fail(c, MESH_ETOOLARGE, "grid too large for this volume shape (at most 2^21 - 31 samples on y)");

    cudaError_t e;
    const size_t es = dtype_size(T);
    const size_t vbytes = (size_t)nx * ny * nz * es;
    c->host_mapped = 0;
    cudaPointerAttributes pa;
    if (vol_on_device) {
        P.vol = vol;
    } else if (p->alg == MESH_ALG_MC && c->zerocopy && cudaPointerGetAttributes(&pa, vol) == cudaSuccess &&
               pa.type == cudaMemoryTypeHost && pa.devicePointer) {
        // pinned and mapped: the one walk reads it in place, once
        P.vol = pa.devicePointer;
        c->host_mapped = 1;
    } else {
        cudaGetLastError();
        if ((e = c->vol.ensure(vbytes)) != cudaSuccess) return cuda_fail(c, e, "volume buffer");
        P.vol = c->vol.ptr;
        if (c->pipe_bytes > 0 && (int64_t)vbytes >= c->pipe_bytes && P.nseg >= 2 && c->tma_env != 1 && !c->one_walk) {
            int rc = ensure_pipe(c);
            if (rc) return rc;
            c->ngroups = std::min(PIPE_MAX, P.nseg);  // the count uploads and classifies
            c->upl_src = vol;
        } else if ((e = cudaMemcpyAsync(c->vol.ptr, vol, vbytes, cudaMemcpyHostToDevice, c->stream)) != cudaSuccess) {
            return cuda_fail(c, e, "volume upload");
        }
    }

    // coordinate tables: xp yp zp dx dy dz (double), the same as float, then the
    // hi/lo float split of the nodes and spacings, computed on the device
    const int64_t ntab = nx + ny + nz;
    if ((e = c->tabs.ensure(table_bytes(ntab))) != cudaSuccess) return cuda_fail(c, e, "table buffer");
    if (c->win_nx && c->win_x0 + nx > c->win_nx) return fail(c, MESH_EINVAL, "volume extends past its x window");
    if ((e = launch_tables((double *)c->tabs.ptr, nx, ny, nz, p->range, L32, c->stream, c->win_x0, c->win_nx)) !=
        cudaSuccess)
        return cuda_fail(c, e, "table launch");
    count_kernels(c, 0, 1);  // the coordinate tables count with the classification
    bind_tables(P, (double *)c->tabs.ptr, nx, ny, nz);
    P.force_fp64 = c->force_fp64;

    // scratch
    const int64_t np = npieces(P);
    P.pstride = np;
    if ((e = c->cnt.ensure((size_t)np * NCNT * sizeof(uint32_t))) != cudaSuccess) return cuda_fail(c, e, "count buffer");
    if ((e = c->base.ensure((size_t)np * NCNT * sizeof(int64_t))) != cudaSuccess) return cuda_fail(c, e, "base buffer");
    const size_t fb = (size_t)P.nchunks * P.tiles_x * P.cy;
    if ((e = c->flags.ensure(fb)) != cudaSuccess) return cuda_fail(c, e, "flag buffer");
    const size_t sb = (scan_scratch_bytes(P) + 255) / 256 * 256;
    if ((e = c->scan.ensure(sb + 64)) != cudaSuccess) return cuda_fail(c, e, "scan buffer");
    P.cnt = (uint32_t *)c->cnt.ptr;
    P.base = (int64_t *)c->base.ptr;
    P.flags = (uint8_t *)c->flags.ptr;
    P.cmask = nullptr;
    if (direct_mc(c)) {
        const size_t mb = (size_t)P.tiles_x * P.cy * P.nchunks * sizeof(uint32_t);
        if ((e = c->cmask.ensure(mb)) != cudaSuccess) return cuda_fail(c, e, "mask buffer");
        P.cmask = (uint32_t *)c->cmask.ptr;
    }
    P.scan_state = (unsigned long long *)c->scan.ptr;
    P.scan_ticket = (unsigned int *)((char *)c->scan.ptr + sb);
    // misc: totals[NCNT] int64, then the error word, the work counter and the
    // staging counter
    P.totals = (int64_t *)c->misc.ptr;
    P.err = (unsigned int *)((int64_t *)c->misc.ptr + NCNT);
    P.work = (unsigned int *)((int64_t *)c->misc.ptr + NCNT + 1);
    P.stage_next = (unsigned long long *)((int64_t *)c->misc.ptr + NCNT + 2);
    P.scan_spin_limit = 1 << 24;
    return MESH_OK;
}

cudaEvent_t take_event(mesh_ctx *c) {
    if (!c->ev_free.empty()) {
        cudaEvent_t e = c->ev_free.back();
        c->ev_free.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return e;
}

// With timing on: kernels launched in `stage` (for mesh_ctx_stage_times).
void count_kernels(mesh_ctx *c, int stage, int n) {
    if (c->timing) c->nkern[stage] += n;
}

void mark(mesh_ctx *c, int stage) {
    if (!c->timing) return;
    cudaEvent_t e = take_event(c);
    if (!e) return;
    cudaEventRecord(e, c->stream);
    c->ev_pairs[stage].push_back(e);
}

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    // thread-safe one-time lookup
    static const PFN_cuTensorMapEncodeTiled_v12000 fn = []() -> PFN_cuTensorMapEncodeTiled_v12000 {
        cudaDriverEntryPointQueryResult q;
        void *f = nullptr;
        const bool ok = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault,
                                                         &q) == cudaSuccess &&
                        q == cudaDriverEntryPointSuccess;
        cudaGetLastError();
        return ok ? (PFN_cuTensorMapEncodeTiled_v12000)f : nullptr;
    }();
    return fn;
}

// Tensor map of the volume for the TMA walk: rows must start on 16-byte
// boundaries and the volume must be at least one box large.
bool make_tensor_map(mesh_ctx *c) {
    const Plan &P = c->plan;
    if (!(c->tma_env == 1 || (c->tma_env < 0 && P.alg == MESH_ALG_MC))) return false;
    int bx;
    size_t es;
    CUtensorMapDataType dt;
    switch (P.T) {
    case MESH_DT_U16: bx = TmaBox<uint16_t>::BX; es = 2; dt = CU_TENSOR_MAP_DATA_TYPE_UINT16; break;
    case MESH_DT_F32: bx = TmaBox<float>::BX; es = 4; dt = CU_TENSOR_MAP_DATA_TYPE_FLOAT32; break;
    case MESH_DT_F64: bx = TmaBox<double>::BX; es = 8; dt = CU_TENSOR_MAP_DATA_TYPE_FLOAT64; break;
    default: return false;  // integer and Float16 volumes take the load walk
    }
    if (((uintptr_t)P.vol & 15) || ((size_t)P.nx * es) % 16 || P.nx < bx || P.ny < TMA_BY || P.nz < TMA_BZ) return false;
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)P.nx, (cuuint64_t)P.ny, (cuuint64_t)P.nz};
    const cuuint64_t strides[2] = {(cuuint64_t)P.nx * es, (cuuint64_t)P.nx * P.ny * es};
    const cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)TMA_BY, (cuuint32_t)TMA_BZ};
    const cuuint32_t elem[3] = {1, 1, 1};
    return enc(&c->tmap, dt, 3, const_cast<void *>(P.vol), dims, strides, box, elem, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
           CUDA_SUCCESS;
}

// Marching Cubes walked once, classification staging the active cells (opt-in;
// also the form that reads a mapped host volume in place).
// (welded meshes need the expansion in emission order, which writes the edge keys)
bool one_walk(const mesh_ctx *c) {
    return c->plan.alg == MESH_ALG_MC && !c->weld && (c->one_walk || c->host_mapped);
}

// Marching Cubes emitted straight from the volume (the default): the classify
// walk leaves per-chunk active-column masks and no list of active cells is
// built (both classify walks write the masks).
bool direct_mc(const mesh_ctx *c) {
    return c->plan.alg == MESH_ALG_MC && !c->list_emit && !one_walk(c);
}

int run_count(mesh_ctx *c) {
    Plan &P = c->plan;
    cudaError_t e;
    if ((e = cudaMemsetAsync(c->misc.ptr, 0, MISC_SLOTS * sizeof(int64_t), c->stream)) != cudaSuccess)
        return cuda_fail(c, e, "memset");
    // the pipelined upload classifies each group with the load walk as it arrives
    c->use_tma = !one_walk(c) && c->ngroups == 1 && make_tensor_map(c);
    mark(c, 0);
    int nlaunch = 1;
    if (one_walk(c)) {
        e = launch_walk_mc(P, c->stream);
    } else if (c->use_tma) {
        e = launch_classify_tma(P, c->tmap, c->stream);
    } else if (c->ngroups > 1) {
        e = upload_and_classify(c);
        nlaunch = c->ngroups;
    } else {
        e = launch_classify(P, c->stream);
    }
    if (e != cudaSuccess) return cuda_fail(c, e, "classify launch");
    mark(c, 0);
    count_kernels(c, 0, nlaunch);
    mark(c, 1);
    if ((e = launch_scan(P, c->stream)) != cudaSuccess) return cuda_fail(c, e, "scan launch");
    mark(c, 1);
    count_kernels(c, 1, 4);  // reduce, column scan, column-sum scan, downsweep
    return MESH_OK;
}

int check_err(mesh_ctx *c) {
    const unsigned err = (unsigned)c->h_misc[NCNT];
    if (err & ERR_SCAN_TIMEOUT) return fail(c, MESH_EDEVICE, "scan look-back wait expired");
    if (err & ERR_TMA_TIMEOUT) return fail(c, MESH_EDEVICE, "TMA stage wait expired");
    if (err & ERR_BOUNDS) return fail(c, MESH_EDEVICE, "device bounds check failed");
    if (err & (ERR_CAPACITY | ERR_STAGE)) return fail(c, MESH_ECAPACITY, "output capacity too small");
    return MESH_OK;
}

int fetch_misc(mesh_ctx *c) {
    cudaError_t e = cudaMemcpyAsync(c->h_misc, c->misc.ptr, MISC_SLOTS * sizeof(int64_t), cudaMemcpyDeviceToHost,
                                    c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "synchronize");
    c->h_misc[NCNT] &= 0xffffffffll;
    return MESH_OK;
}

// List of active cells (Marching Cubes), room for `cap` entries.
int ensure_entries(mesh_ctx *c, int64_t cap) {
    Plan &P = c->plan;
    const size_t es = dtype_size(P.T);
    const int64_t nside = cap / ENT_BLOCK + 1;
    auto up = [](size_t n) { return (n + 255) / 256 * 256; };  // every array 256-byte aligned
    const size_t o_val = up((size_t)cap * 8);
    const size_t o_side = o_val + up((size_t)cap * 8 * es);
    const size_t o_rank = o_side + up((size_t)nside * 16);
    const size_t o_cs = o_rank + up((size_t)cap * 8);
    const size_t bytes = o_cs + up((size_t)cap + 1);
    cudaError_t e = c->ent.ensure(bytes);
    if (e != cudaSuccess) return cuda_fail(c, e, "entry buffer");
    char *b = (char *)c->ent.ptr;
    P.ent_pos = (unsigned long long *)b;
    P.ent_val = b + o_val;  // 8 corner values per entry (vector stores need 16-byte alignment)
    P.ent_side = (long long *)(b + o_side);
    P.ent_rank = (uint2 *)(b + o_rank);
    P.ent_cs = (uint8_t *)(b + o_cs);
    P.ent_cap = cap;
    c->ent_cap_seen = std::max(c->ent_cap_seen, cap);
    return MESH_OK;
}

int launch_emit(mesh_ctx *c) {
    cudaError_t e;
    if (one_walk(c)) {
        mark(c, 3);
        e = launch_expand_staged_mc(c->plan, c->Q64, c->P64, c->stream);
        mark(c, 3);
        count_kernels(c, 3, 1);
        return e != cudaSuccess ? cuda_fail(c, e, "expand launch") : MESH_OK;
    }
    if (direct_mc(c)) {
        mark(c, 2);
        e = launch_direct_mc(c->plan, c->Q64, c->P64, c->stream);
        mark(c, 2);
        count_kernels(c, 2, 1);
        return e != cudaSuccess ? cuda_fail(c, e, "emit launch") : MESH_OK;
    }
    mark(c, 2);
    if (c->plan.alg == MESH_ALG_MC) e = launch_emit_mc(c->plan, c->Q64, c->P64, 0, c->stream);
    else e = launch_emit_halo(c->plan, c->Q64, c->A64, c->P64, c->stream);
    mark(c, 2);
    count_kernels(c, 2, 1);
    if (e != cudaSuccess) return cuda_fail(c, e, "emit launch");
    if (c->plan.alg == MESH_ALG_MC) {
        mark(c, 3);
        e = launch_emit_mc(c->plan, c->Q64, c->P64, 1, c->stream);
        mark(c, 3);
        count_kernels(c, 3, 1);
        if (e != cudaSuccess) return cuda_fail(c, e, "expand launch");
    }
    return MESH_OK;
}

// Marching Cubes emission into host buffers in K x ranges of whole x tiles.  The
// emission order is x-major, so the cells of an x range own one contiguous run of
// list entries, vertices and faces, starting at the scanned base of the range's
// first piece (seg 0, y 0, x0).  Range g is compacted and expanded on the compute
// stream; its vertices and faces go down on the copy stream while range g + 1 is
// emitted.  All launches are enqueued before the copies, so a pageable (blocking)
// destination still overlaps the copies with the emission.
int emit_pipelined(mesh_ctx *c, int K, void *verts, int64_t *faces) {
    const Plan &P = c->plan;
    const int64_t np = P.pstride;
    const size_t vsz = (size_t)3 * (P.out64 ? 8 : 4);
    int tx[PIPE_MAX + 1];
    for (int g = 0; g <= K; g++) tx[g] = (int)((int64_t)g * P.tiles_x / K);
    GatherIdx gi{};
    gi.n = 3 * (K - 1);
    for (int g = 1; g < K; g++) {
        const int64_t i = piece(P, 0, 0, tx[g] * TILE_X);
        for (int k = 0; k < 3; k++) gi.idx[3 * (g - 1) + k] = k * np + i;
    }
    cudaError_t e = launch_gather(P.base, gi, (int64_t *)c->gat.ptr, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(c->h_gat, c->gat.ptr, (size_t)gi.n * sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "split points");
    int64_t V[PIPE_MAX + 1], F[PIPE_MAX + 1], E[PIPE_MAX + 1];
    V[0] = F[0] = E[0] = 0;
    V[K] = c->nverts;
    F[K] = c->nfaces;
    E[K] = c->nactive;
    for (int g = 1; g < K; g++) {
        V[g] = c->h_gat[3 * (g - 1)];
        F[g] = c->h_gat[3 * (g - 1) + 1];
        E[g] = c->h_gat[3 * (g - 1) + 2];
    }
    for (int g = 0; g < K; g++)
        if (V[g] > V[g + 1] || F[g] > F[g + 1] || E[g] > E[g + 1] || V[g + 1] > c->nverts || F[g + 1] > c->nfaces)
            return fail(c, MESH_EDEVICE, "inconsistent split points");
    int nexp = 0;
    mark(c, 2);
    for (int g = 0; g < K && e == cudaSuccess; g++) {
        Plan q = P;
        q.tx0 = tx[g];
        q.ntx = tx[g + 1] - tx[g];
        q.e_lo = E[g];
        q.e_hi = E[g + 1];
        if (direct_mc(c)) {
            e = launch_direct_mc(q, c->Q64, c->P64, c->stream);
        } else {
            e = launch_emit_mc(q, c->Q64, c->P64, 0, c->stream);
            if (e == cudaSuccess && E[g + 1] > E[g]) {
                e = launch_emit_mc(q, c->Q64, c->P64, 1, c->stream);
                nexp++;
            }
        }
        if (e == cudaSuccess) e = cudaEventRecord(c->ev_part[g], c->stream);
    }
    mark(c, 2);
    count_kernels(c, 2, K);
    count_kernels(c, 3, nexp);
    if (e != cudaSuccess) return cuda_fail(c, e, "emit launch");
    for (int g = 0; g < K && e == cudaSuccess; g++) {
        e = cudaStreamWaitEvent(c->copy, c->ev_part[g], 0);
        if (e == cudaSuccess && V[g + 1] > V[g])
            e = cudaMemcpyAsync((char *)verts + V[g] * vsz, (const char *)P.verts + V[g] * vsz,
                                (size_t)(V[g + 1] - V[g]) * vsz, cudaMemcpyDeviceToHost, c->copy);
        if (e == cudaSuccess && F[g + 1] > F[g])
            e = cudaMemcpyAsync(faces + 3 * F[g], P.faces + 3 * F[g], (size_t)(F[g + 1] - F[g]) * 24,
                                cudaMemcpyDeviceToHost, c->copy);
    }
    if (e == cudaSuccess) e = cudaEventRecord(c->ev_done, c->copy);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->stream, c->ev_done, 0);
    return e != cudaSuccess ? cuda_fail(c, e, "mesh download") : MESH_OK;
}

// Staging slots of the one walk beyond its active cells: at most a block per warp.
int64_t stage_slack(const Plan &P) { return (int64_t)STG_BLK * P.tiles_x * P.tiles_y * P.nseg; }

bool degenerate(int64_t nx, int64_t ny, int64_t nz) { return nx < 2 || ny < 2 || nz < 2; }

}  // namespace

extern "C" {

void mesh_params_default(mesh_params *p) {
    if (!p) return;
    memset(p, 0, sizeof(*p));
    p->alg = MESH_ALG_MC;
    p->iso_type = MESH_DT_F64;
    p->iso = 0.0;
    p->eps_type = MESH_DT_F64;
    p->eps = 1e-3;
    p->range_type = MESH_DT_I64;
    p->range[0] = p->range[2] = p->range[4] = -1.0;
    p->range[1] = p->range[3] = p->range[5] = 1.0;
}

const char *mesh_status_string(int s) {
    switch (s) {
    case MESH_OK: return "ok";
    case MESH_EINVAL: return "invalid argument";
    case MESH_ENOMEM: return "out of memory";
    case MESH_ECUDA: return "CUDA error";
    case MESH_EDEVICE: return "device-side error";
    case MESH_ESTATE: return "mesh_fill called without a successful mesh_count";
    case MESH_ECAPACITY: return "output capacity too small";
    case MESH_ETOOLARGE: return "volume too large";
    case MESH_ESCRATCH: return "needs more scratch than the no-allocation limit";
    case MESH_EBUDGET: return "worst case exceeds the memory budget";
    case MESH_EBUSY: return "queue full";
    default: return "unknown status";
    }
}

const char *mesh_ctx_last_error(const mesh_ctx *c) { return c ? c->msg.c_str() : ""; }

int mesh_ctx_create(int device, mesh_ctx **out) {
    if (!out) return MESH_EINVAL;
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || device < 0 || device >= n) {
        cudaGetLastError();
        return e != cudaSuccess ? MESH_ECUDA : MESH_EINVAL;
    }
    if ((e = cudaSetDevice(device)) != cudaSuccess) return MESH_ECUDA;
    mesh_ctx *c = new (std::nothrow) mesh_ctx();
    if (!c) return MESH_ENOMEM;
    c->device = device;
    cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device);
    if (cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking) != cudaSuccess ||
        c->misc.ensure(MISC_SLOTS * sizeof(int64_t)) != cudaSuccess ||
        cudaHostAlloc((void **)&c->h_misc, MISC_SLOTS * sizeof(int64_t), cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        mesh_ctx_destroy(c);
        return MESH_ENOMEM;
    }
    c->stream = c->own;
    const char *ff = getenv("MESHING_GB300_FORCE_FP64");
    c->force_fp64 = ff && ff[0] == '1';
    const char *wt = getenv("MESHING_GB300_TMA");
    c->tma_env = (wt && wt[0] == '1') ? 1 : (wt && wt[0] == '0') ? 0 : -1;
    const char *ow = getenv("MESHING_GB300_ONE_WALK");
    c->one_walk = ow && ow[0] == '1';
    const char *le = getenv("MESHING_GB300_LIST_EMIT");
    c->list_emit = le && le[0] == '1';
    const char *zc = getenv("MESHING_GB300_ZEROCOPY");
    c->zerocopy = zc && zc[0] == '1';
    const char *pb = getenv("MESHING_GB300_PIPELINE_BYTES");  // <= 0: never pipelined
    if (pb && pb[0]) c->pipe_bytes = strtoll(pb, nullptr, 10);
    *out = c;
    return MESH_OK;
}

void mesh_ctx_destroy(mesh_ctx *c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->copy) cudaStreamSynchronize(c->copy);
    DevBuf *bufs[] = {&c->vol,   &c->tabs,  &c->cnt, &c->base, &c->flags,    &c->scan,   &c->misc,
                      &c->out_v, &c->out_f, &c->ent, &c->nrm,  &c->weld_buf, &c->weld_v, &c->gat,
                      &c->cmask};
    for (DevBuf *b : bufs) b->release();
    for (cudaEvent_t e : c->ev_part)
        if (e) cudaEventDestroy(e);
    if (c->ev_ready) cudaEventDestroy(c->ev_ready);
    if (c->ev_done) cudaEventDestroy(c->ev_done);
    if (c->copy) cudaStreamDestroy(c->copy);
    if (c->h_gat) cudaFreeHost(c->h_gat);
    for (auto &v : c->ev_pairs)
        for (cudaEvent_t e : v) cudaEventDestroy(e);
    for (cudaEvent_t e : c->ev_free) cudaEventDestroy(e);
    if (c->h_misc) cudaFreeHost(c->h_misc);
    if (c->own) cudaStreamDestroy(c->own);
    delete c;
}

int mesh_ctx_set_stream(mesh_ctx *c, void *stream) {
    if (!c) return MESH_EINVAL;
    c->stream = stream ? (cudaStream_t)stream : c->own;
    return MESH_OK;
}

int mesh_set_x_window(mesh_ctx *c, int64_t x_first, int64_t nx_total, int halo) {
    if (!c) return MESH_EINVAL;
    if (x_first < 0 || nx_total < 0 || (nx_total == 0 && (x_first != 0 || halo)) ||
        nx_total > ((int64_t)1 << POS_BITS) || (halo != 0 && halo != 1))
        return fail(c, MESH_EINVAL, "invalid x window");
    c->win_x0 = x_first;
    c->win_nx = nx_total;
    c->win_halo = halo;
    c->have_plan = 0;
    return MESH_OK;
}

int mesh_output_float_bits(int T, const mesh_params *p, int *bits) {
    if (!p || !bits) return MESH_EINVAL;
    int rc = validate(nullptr, T, 0, 0, 0, p);
    if (rc) return rc;
    const int tys[4] = {p->range_type, T, p->iso_type, p->eps_type};
    *bits = out_is_f64(tys, p->alg == MESH_ALG_MT ? 4 : 3) ? 64 : 32;
    return MESH_OK;
}

// Welded Marching Cubes: extract the per-cell mesh with its edge keys into the
// context's buffers, weld it (k_weld.cu) and keep the welded counts.
int run_weld(mesh_ctx *c) {
    Plan &P = c->plan;
    const int64_t nv = c->nverts, nf = c->nfaces;
    const size_t es = P.out64 ? 8 : 4;
    const int64_t nb = weld_blocks(nv), hcap = weld_hash_slots(nv);
    auto up = [](size_t n) { return (n + 255) / 256 * 256; };
    const size_t o_bsum = up((size_t)nv * 8), o_hkey = o_bsum + up((size_t)(nb + 1) * 8),
                 o_hval = o_hkey + up((size_t)hcap * 8), total = o_hval + up((size_t)hcap * 8);
    cudaError_t e;
    if ((e = c->out_v.ensure((size_t)nv * 3 * es + 16)) != cudaSuccess) return cuda_fail(c, e, "vertex buffer");
    if ((e = c->out_f.ensure((size_t)nf * 24 + 16)) != cudaSuccess) return cuda_fail(c, e, "face buffer");
    if ((e = c->weld_v.ensure((size_t)nv * 3 * es + 16)) != cudaSuccess) return cuda_fail(c, e, "welded vertices");
    if ((e = c->weld_buf.ensure(total)) != cudaSuccess) return cuda_fail(c, e, "weld scratch");
    char *wb = (char *)c->weld_buf.ptr;
    P.verts = c->out_v.ptr;
    P.faces = (int64_t *)c->out_f.ptr;
    P.verts_cap = nv;
    P.faces_cap = nf;
    P.vkey = (long long *)wb;
    int rc;
    if (!direct_mc(c) && (rc = ensure_entries(c, c->nactive))) return rc;
    if ((e = cudaMemsetAsync(P.err, 0, sizeof(unsigned), c->stream)) != cudaSuccess) return cuda_fail(c, e, "memset");
    if ((rc = launch_emit(c))) return rc;
    if ((e = launch_weld(P.vkey, nv, P.verts, P.out64, P.faces, nf, (long long *)(wb + o_bsum), c->weld_v.ptr,
                         (unsigned long long *)(wb + o_hkey), (long long *)(wb + o_hval), hcap, P.err, c->sms,
                         c->stream)) != cudaSuccess)
        return cuda_fail(c, e, "weld launch");
    long long nw = 0;
    if ((e = cudaMemcpyAsync(&nw, wb + o_bsum + (size_t)nb * 8, 8, cudaMemcpyDeviceToHost, c->stream)) != cudaSuccess)
        return cuda_fail(c, e, "welded count");
    if ((rc = fetch_misc(c))) return rc;  // synchronizes
    if ((rc = check_err(c))) return rc;
    c->nverts = nw;
    P.vkey = nullptr;
    return MESH_OK;
}

}  // extern "C"

namespace {
// An x window with a halo column (MT / NSN slab after the first): the halo
// column's vertices and faces come first in the scan and are not emitted, so
// the counts lose its totals (the scanned base of piece (seg 0, y 0, x 1)).
int drop_halo_counts(mesh_ctx *c) {
    const Plan &P = c->plan;
    int64_t v0 = c->nverts, f0 = c->nfaces;  // a window of the halo column alone emits nothing
    if (P.cx > 1) {
        GatherIdx gi{};
        gi.n = 2;
        gi.idx[0] = piece(P, 0, 0, 1);
        gi.idx[1] = P.pstride + piece(P, 0, 0, 1);
        cudaError_t e = c->gat.ensure(GATHER_MAX * sizeof(int64_t));
        if (e == cudaSuccess) e = launch_gather(P.base, gi, (int64_t *)c->gat.ptr, c->stream);
        int64_t h[2] = {0, 0};
        if (e == cudaSuccess) e = cudaMemcpyAsync(h, c->gat.ptr, sizeof(h), cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) return cuda_fail(c, e, "halo counts");
        v0 = h[0];
        f0 = h[1];
    }
    if (v0 < 0 || v0 > c->nverts || f0 < 0 || f0 > c->nfaces) return fail(c, MESH_EDEVICE, "inconsistent halo counts");
    c->nverts -= v0;
    c->nfaces -= f0;
    return MESH_OK;
}
}  // namespace

extern "C" {

int mesh_count(mesh_ctx *c, const void *vol, int T, int64_t nx, int64_t ny, int64_t nz, int vol_on_device,
               const mesh_params *p, int64_t *nverts, int64_t *nfaces) {
    if (!c || !nverts || !nfaces) return fail(c, MESH_EINVAL, "NULL argument");
    c->have_plan = 0;
    c->msg.clear();
    int rc = validate(c, T, nx, ny, nz, p);
    if (rc) return rc;
    if (cudaSetDevice(c->device) != cudaSuccess) return fail(c, MESH_ECUDA, "cudaSetDevice");
    if (degenerate(nx, ny, nz)) {
        c->nverts = c->nfaces = 0;
        c->plan = Plan{};
        c->plan.alg = p->alg;
        c->have_plan = 2;  // empty mesh
        *nverts = *nfaces = 0;
        return MESH_OK;
    }
    if (!vol) return fail(c, MESH_EINVAL, "volume is NULL");
    if ((rc = prepare(c, vol, T, nx, ny, nz, vol_on_device, p))) return rc;
    if (one_walk(c)) {
        // the list of active cells is filled during the count: start from a
        // guess (or the context's earlier list), and if the walk ran out of
        // slots walk again with the exact number it reported
        const int64_t cells = (int64_t)c->plan.cx * c->plan.cy * c->plan.cz;
        const int64_t guess = std::max<int64_t>(c->ent_cap_seen, cells / 48 + stage_slack(c->plan));
        if ((rc = ensure_entries(c, guess))) return rc;
    }
    if ((rc = run_count(c))) return rc;
    if ((rc = fetch_misc(c))) return rc;
    if (one_walk(c) && ((unsigned)c->h_misc[NCNT] & ERR_STAGE)) {
        if ((rc = ensure_entries(c, c->h_misc[NCNT + 2]))) return rc;
        if ((rc = run_count(c))) return rc;
        if ((rc = fetch_misc(c))) return rc;
    }
    if ((rc = check_err(c))) return rc;
    c->nverts = c->h_misc[0];
    c->nfaces = c->h_misc[1];
    c->nactive = c->h_misc[2];
    if (c->plan.xhalo && (rc = drop_halo_counts(c))) return rc;
    if (c->weld && (rc = run_weld(c))) return rc;
    *nverts = c->nverts;
    *nfaces = c->nfaces;
    c->have_plan = 1;
    return MESH_OK;
}

int mesh_fill(mesh_ctx *c, void *verts, int64_t *faces, int out_on_device) {
    if (!c) return MESH_EINVAL;
    if (!c->have_plan) return fail(c, MESH_ESTATE, "mesh_fill without mesh_count");
    if (c->have_plan == 2 || (c->nverts == 0 && c->nfaces == 0)) return MESH_OK;
    if ((c->nverts && !verts) || (c->nfaces && !faces)) return fail(c, MESH_EINVAL, "NULL output");
    if (cudaSetDevice(c->device) != cudaSuccess) return fail(c, MESH_ECUDA, "cudaSetDevice");
    Plan &P = c->plan;
    const size_t vb = (size_t)c->nverts * 3 * (P.out64 ? 8 : 4), fbytes = (size_t)c->nfaces * 3 * 8;
    cudaError_t e;
    if (c->weld) {  // the welded mesh was built by the count: copy it out
        const cudaMemcpyKind k = out_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
        if (vb && (e = cudaMemcpyAsync(verts, c->weld_v.ptr, vb, k, c->stream)) != cudaSuccess)
            return cuda_fail(c, e, "welded vertex copy");
        if (fbytes && (e = cudaMemcpyAsync(faces, c->out_f.ptr, fbytes, k, c->stream)) != cudaSuccess)
            return cuda_fail(c, e, "welded face copy");
        if ((e = cudaStreamSynchronize(c->stream)) != cudaSuccess) return cuda_fail(c, e, "synchronize");
        c->have_plan = 0;
        return MESH_OK;
    }
    if (out_on_device) {
        P.verts = verts;
        P.faces = faces;
    } else {
        if ((e = c->out_v.ensure(vb + 16)) != cudaSuccess) return cuda_fail(c, e, "vertex staging");
        if ((e = c->out_f.ensure(fbytes + 16)) != cudaSuccess) return cuda_fail(c, e, "face staging");
        P.verts = c->out_v.ptr;
        P.faces = (int64_t *)c->out_f.ptr;
    }
    P.verts_cap = c->nverts;
    P.faces_cap = c->nfaces;
    int rc;
    if (P.alg == MESH_ALG_MC && !one_walk(c) && !direct_mc(c) && (rc = ensure_entries(c, c->nactive))) return rc;
    if ((e = cudaMemsetAsync(P.err, 0, sizeof(unsigned), c->stream)) != cudaSuccess) return cuda_fail(c, e, "memset");
    int parts = 1;
    if (!out_on_device && P.alg == MESH_ALG_MC && !one_walk(c) && c->pipe_bytes > 0 &&
        (int64_t)(vb + fbytes) >= c->pipe_bytes && P.tiles_x >= 2) {
        if ((rc = ensure_pipe(c))) return rc;
        parts = std::min(PIPE_MAX, P.tiles_x);
    }
    if (parts > 1) {
        if ((rc = emit_pipelined(c, parts, verts, faces))) return rc;
    } else {
        if ((rc = launch_emit(c))) return rc;
        if (!out_on_device) {
            if (vb && (e = cudaMemcpyAsync(verts, P.verts, vb, cudaMemcpyDeviceToHost, c->stream)) != cudaSuccess)
                return cuda_fail(c, e, "vertex download");
            if (fbytes &&
                (e = cudaMemcpyAsync(faces, P.faces, fbytes, cudaMemcpyDeviceToHost, c->stream)) != cudaSuccess)
                return cuda_fail(c, e, "face download");
        }
    }
    if ((rc = fetch_misc(c))) return rc;
    c->have_plan = 0;  // a plan may reference a caller's device volume: one fill per count
    return check_err(c);
}

int mesh_extract_device(mesh_ctx *c, const void *vol, int T, int64_t nx, int64_t ny, int64_t nz,
                        const mesh_params *p, void *verts, int64_t verts_cap, int64_t *faces, int64_t faces_cap,
                        int64_t *counts) {
    if (!c || !counts) return fail(c, MESH_EINVAL, "NULL argument");
    c->msg.clear();
    int rc = validate(c, T, nx, ny, nz, p);
    if (rc) return rc;
    if (cudaSetDevice(c->device) != cudaSuccess) return fail(c, MESH_ECUDA, "cudaSetDevice");
    cudaError_t e;
    if (degenerate(nx, ny, nz)) {
        if ((e = cudaMemsetAsync(counts, 0, 2 * sizeof(int64_t), c->stream)) != cudaSuccess)
            return cuda_fail(c, e, "memset");
        return MESH_OK;
    }
    if (!vol) return fail(c, MESH_EINVAL, "volume is NULL");
    if (p->alg == MESH_ALG_MC_WELDED) return fail(c, MESH_EINVAL, "welded meshes are built by mesh_count / mesh_fill");
    if ((rc = prepare(c, vol, T, nx, ny, nz, 1, p))) return rc;
    Plan &P = c->plan;
    if (P.xhalo) return fail(c, MESH_EINVAL, "an x window with a halo column is meshed by mesh_count / mesh_fill");
    P.verts = verts;
    P.faces = faces;
    P.verts_cap = verts ? verts_cap : 0;
    P.faces_cap = faces ? faces_cap : 0;
    // an active Marching Cubes cell emits at least 3 vertices; the one walk
    // also leaves up to a block of slots per warp unused
    if (P.alg == MESH_ALG_MC && !direct_mc(c) &&
        (rc = ensure_entries(c, P.verts_cap / 3 + (one_walk(c) ? stage_slack(P) : 0))))
        return rc;
    if ((rc = run_count(c))) return rc;
    if ((rc = launch_emit(c))) return rc;
    if ((e = cudaMemcpyAsync(counts, P.totals, 2 * sizeof(int64_t), cudaMemcpyDeviceToDevice, c->stream)) !=
        cudaSuccess)
        return cuda_fail(c, e, "count copy");
    c->have_plan = 0;
    return MESH_OK;
}

int mesh_ctx_sync(mesh_ctx *c) {
    if (!c) return MESH_EINVAL;
    if (cudaSetDevice(c->device) != cudaSuccess) return fail(c, MESH_ECUDA, "cudaSetDevice");
    int rc = fetch_misc(c);
    if (rc) return rc;
    return check_err(c);
}

int mesh_ctx_enable_timing(mesh_ctx *c, int enable) {
    if (!c) return MESH_EINVAL;
    c->timing = enable ? 1 : 0;
    return MESH_OK;
}

int mesh_ctx_stage_times(mesh_ctx *c, double *ms, int64_t *launches) {
    if (!c || !ms || !launches) return MESH_EINVAL;
    if (cudaSetDevice(c->device) != cudaSuccess) return fail(c, MESH_ECUDA, "cudaSetDevice");
    int rc = MESH_OK;
    for (int s = 0; s < NSTAGE; s++) {
        ms[s] = 0;
        launches[s] = 0;
        auto &v = c->ev_pairs[s];
        for (size_t i = 0; i + 1 < v.size(); i += 2) {
            float t = 0;
            cudaError_t e = cudaEventSynchronize(v[i + 1]);
            if (e == cudaSuccess) e = cudaEventElapsedTime(&t, v[i], v[i + 1]);
            if (e != cudaSuccess) rc = cuda_fail(c, e, "stage timing");
            ms[s] += t;
        }
        launches[s] = c->nkern[s];
        c->nkern[s] = 0;
        for (cudaEvent_t e : v) c->ev_free.push_back(e);
        v.clear();
    }
    return rc;
}

}  // extern "C"
