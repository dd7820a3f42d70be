// Serving loop behind the C ABI (mesh_server_* in include/meshing_gb300.h).
//
// No counterpart in the reference, which answers one isosurface() call at a
// time.  Requests (a volume in device or host memory, its shape and the
// algorithm parameters) arrive on any thread and wait in a FIFO queue.  A loop thread
// admits them by continuous batching: whenever one of the server's wave slots
// is free it takes queued requests in order while the device pool can reserve
// each one's worst-case vertex / face output (and the wave's scratch), and
// launches them together as one wave on the slot's stream:
//   * Marching Cubes requests with the same volume type and iso run as one
//     batch (k_classify_batch .. k_expand_mc<EXP_BATCH>) that writes every
//     volume's mesh straight into that request's own output block;
//   * Marching Tetrahedra and Naive Surface Nets requests run the
//     single-volume kernels on the slot's context, into their output blocks;
//   * welded Marching Cubes requests run the slot context's welded extraction
//     (the Marching Cubes kernels, then the weld, in the context's own scratch)
//     and their welded mesh is copied into their output blocks.
// A host volume gets a block of the pool for itself at admission (counted
// against the budget like the outputs), is uploaded on the slot's stream ahead
// of its wave's kernels and gives the block back when the wave's results are
// published.
// Waves on different slots overlap on the device.  A host function queued
// after the wave's kernels stamps the completion time, publishes the counts
// and frees the wave's scratch; a request's output block stays reserved, and
// its mesh resident, until the client releases it.  Each request's mesh is
// exactly the one isosurface() returns for it alone.
//
// Worst-case bounds per request (cells = (nx-1)(ny-1)(nz-1), nodes = nx ny nz):
//   Marching Cubes      12 vertices and 5 faces per cell (the largest cases)
//   Marching Tetrahedra 7 vertices per node (the 7 edge directions a node owns),
//                       12 faces per cell (6 tetrahedra, 2 triangles each)
//   Naive Surface Nets  1 vertex per cell, 2 faces per crossed base edge (3 per node)
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "mesh_host.h"
#include "mesh_internal.cuh"

using namespace mesh;

namespace {

using clk = std::chrono::steady_clock;
constexpr size_t GRAIN = 256;
constexpr int MAX_GROUPS = 4;  // Marching Cubes batches per wave (distinct volume type / iso)
constexpr size_t GROUP_FIXED_BYTES = 16 * 256 + 256 + 64;

size_t up(size_t n) { return (n + GRAIN - 1) / GRAIN * GRAIN; }

struct Block {
    size_t off = 0, size = 0;
};

// First-fit allocator over the device arena; host bookkeeping only.
struct Pool {
    size_t cap = 0, used = 0, peak = 0;
    std::map<size_t, size_t> free_;  // offset -> size
    void init(size_t c) {
        cap = c / GRAIN * GRAIN;
        free_.clear();
        if (cap) free_[0] = cap;
        used = peak = 0;
    }
    bool alloc(size_t n, Block *b) {
        n = up(std::max<size_t>(n, 1));
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < n) continue;
            const size_t o = it->first, rest = it->second - n;
            free_.erase(it);
            if (rest) free_[o + n] = rest;
            b->off = o;
            b->size = n;
            used += n;
            peak = std::max(peak, used);
            return true;
        }
        return false;
    }
    // The same from the top of the highest free chunk that fits (finished meshes
    // are kept there, away from the worst-case blocks of requests in flight).
    bool alloc_top(size_t n, Block *b) {
        n = up(std::max<size_t>(n, 1));
        for (auto it = free_.rbegin(); it != free_.rend(); ++it) {
            if (it->second < n) continue;
            const size_t o = it->first, sz = it->second;
            free_.erase(std::next(it).base());
            if (sz > n) free_[o] = sz - n;
            b->off = o + sz - n;
            b->size = n;
            used += n;
            peak = std::max(peak, used);
            return true;
        }
        return false;
    }
    // Frees [o, o + n) of an allocated block (both multiples of GRAIN).
    void release_range(size_t o, size_t n) {
        if (!n) return;
        Block b;
        b.off = o;
        b.size = n;
        release(&b);
    }
    size_t largest() const {
        size_t m = 0;
        for (auto &f : free_) m = std::max(m, f.second);
        return m;
    }
    void release(Block *b) {
        if (!b->size) return;
        used -= b->size;
        size_t o = b->off, n = b->size;
        auto nx = free_.lower_bound(o);
        if (nx != free_.end() && o + n == nx->first) {
            n += nx->second;
            nx = free_.erase(nx);
        }
        if (nx != free_.begin()) {
            auto pv = std::prev(nx);
            if (pv->first + pv->second == o) {
                o = pv->first;
                n += pv->second;
                free_.erase(pv);
            }
        }
        free_[o] = n;
        b->size = 0;
    }
};

enum { RQ_QUEUED = 0, RQ_RUNNING = 1, RQ_DONE = 2, RQ_FAILED = 3 };

struct Req {
    int64_t id = 0;
    const void *vol = nullptr;        // device volume (for a host request: its pool copy, once uploaded)
    const void *host_vol = nullptr;   // host volume of a host request
    size_t vol_bytes = 0;             // bytes of a host request's volume
    Block vin;                        // its pool copy while the request is in flight
    int T = 0;
    int64_t dims[3] = {0, 0, 0};
    mesh_params p{};
    int out64 = 0;
    int64_t vcap = 0, fcap = 0;
    size_t vbytes = 0;  // bytes of the vertex part of the output block
    Block out;          // worst case while in flight: vertices at 0, faces at vbytes
    Block keep_v, keep_f;  // after completion: the blocks holding the mesh
    Block move_v, move_f;  // while the mesh is being moved: where it goes
    int state = RQ_QUEUED;
    int status = MESH_OK;
    int64_t nverts = 0, nfaces = 0;
    clk::time_point t_sub, t_done;
};

struct Group {  // one Marching Cubes batch of a wave
    int T = 0, iso_type = 0, range_type = 0;
    double iso = 0;
    std::vector<int64_t> reqs;
    size_t bound = GROUP_FIXED_BYTES;  // upper bound of the scratch (GROUP_FIXED + shares)
    Block scratch;
    size_t res_off = 0;    // first result word in the slot's pinned results
    size_t stage_off = 0;  // the batch's head in the slot's pinned staging
};

struct Slot {
    mesh_server *srv = nullptr;
    int index = 0;
    cudaStream_t stream = nullptr;
    mesh_ctx *ctx = nullptr;       // Marching Tetrahedra / Naive Surface Nets requests
    int busy = 0;
    int launching = 0;             // the loop thread is queuing this slot's wave
    char *stage = nullptr;         // pinned staging of batch plans
    size_t stage_cap = 0;
    int64_t *res = nullptr;        // pinned results: counts and error words
    size_t res_cap = 0;            // in int64 words
    int64_t *d_counts = nullptr;   // device counts of the single-volume requests
    size_t d_counts_cap = 0;
    std::vector<Group> groups;
    std::vector<int64_t> singles;  // single-volume requests of the wave
    size_t single_res_off = 0;
    // copies of the wave's requests, taken under the lock at admission: the
    // launch reads these, never the server's request map, which other threads
    // grow (and rehash) while a wave is being queued
    std::unordered_map<int64_t, Req> wave;
    uint64_t seq = 0;  // waves launched on this slot
    int finishing = 0; // the wave's kernels are done; its meshes still have to be moved
};

// Argument of a wave's host function: the slot and which of its waves.
struct WaveTag {
    Slot *sl;
    uint64_t seq;
};

// Scratch of a Marching Cubes batch laid out in one block.
struct GroupLayout {
    BatchSizes z;
    std::vector<BatchVol> hv;
    std::vector<int64_t> tab_off;
    size_t o_ivol = 0, o_svol = 0, o_jobs = 0, head = 0;  // head: copied from pinned staging
    size_t o_tabs = 0, o_cnt = 0, o_base = 0, o_flags = 0, o_scan = 0, o_misc = 0, o_offs = 0;
    size_t o_pos = 0, o_val = 0, o_side = 0, o_vol = 0, o_cs = 0, total = 0;
    int64_t cells = 0;
    bool scan_vol = false;  // the per-volume scan (every volume at most 128 columns wide)
};


void layout_group(const std::vector<const Req *> &rs, GroupLayout *L) {
    const int n = (int)rs.size();
    std::vector<int64_t> dims(3 * (size_t)n);
    L->cells = 0;
    for (int i = 0; i < n; i++) {
        for (int k = 0; k < 3; k++) dims[3 * i + k] = rs[i]->dims[k];
        if (dims[3 * i] > 1 && dims[3 * i + 1] > 1 && dims[3 * i + 2] > 1)
            L->cells += (dims[3 * i] - 1) * (dims[3 * i + 1] - 1) * (dims[3 * i + 2] - 1);
    }
    L->z = tile_batch(dims.data(), n, 0, L->hv, L->tab_off);
    // every volume at most 4 column groups wide: one scan CTA per volume, chained
    L->scan_vol = n > 0;
    for (const BatchVol &bv : L->hv) L->scan_vol = L->scan_vol && bv.cx <= 4 * 32;
    const BatchSizes &z = L->z;
    const size_t es = n ? dtype_size(rs[0]->T) : 4;
    size_t o = up(sizeof(BatchVol) * (size_t)std::max(n, 1));
    L->o_ivol = o; o += up(4 * (size_t)z.items + 4);
    L->o_svol = o; o += up(4 * (size_t)z.stiles + 4);
    L->o_jobs = o; o += up(sizeof(TabJob) * (size_t)std::max(n, 1));
    L->head = o;
    L->o_tabs = o; o += up(8 * (size_t)z.tdoubles + 8);
    L->o_cnt = o; o += up((size_t)z.pieces * NCNT * 4 + 4);
    L->o_base = o; o += up((size_t)z.pieces * NCNT * 8 + 8);
    L->o_flags = o; o += up((size_t)z.nflags + 1);
    L->o_scan = o; o += up((size_t)std::max<int64_t>(z.stiles, n) * NCNT * 8 + 64);
    L->o_misc = o; o += up(MISC_SLOTS * 8);
    L->o_offs = o; o += up((size_t)(n + 1) * 16);
    const size_t cap = (size_t)L->cells;  // worst case: every cell active
    L->o_pos = o; o += up(cap * 8 + 8);
    L->o_val = o; o += up(cap * 8 * es + 16);
    L->o_side = o; o += up((cap / ENT_BLOCK + 1) * 16);
    L->o_vol = o; o += up(cap * 4 + 4);
    L->o_cs = o; o += up(cap + 1);
    L->total = o;
}

// An upper bound of volume r's share of a batch's scratch: every array of
// layout_group grows by at most this much when r joins (before rounding).
size_t vol_scratch_bytes(const Req &r) {
    const int64_t nx = r.dims[0], ny = r.dims[1], nz = r.dims[2];
    size_t b = sizeof(BatchVol) + sizeof(TabJob) + 16 + 4 + 4 + 8 + NCNT * 8;
    if (nx > 1 && ny > 1 && nz > 1) {
        const int64_t cx = nx - 1, cy = ny - 1, cz = nz - 1, cells = cx * cy * cz;
        const int64_t zs = (cz + ZC - 1) / ZC * ZC;
        const int64_t tx = (cx + TILE_X - 1) / TILE_X, ty = (cy + WY - 1) / WY, st = (cx + 31) / 32;
        b += 4 * (size_t)(tx * ty) + 4 * (size_t)st + table_bytes(nx + ny + nz) + 256;
        b += (size_t)cy * cx * NCNT * (4 + 8) + (size_t)(zs / ZC) * tx * cy + (size_t)st * NCNT * 8;
        b += (size_t)cells * (8 + 8 * dtype_size(r.T) + 4 + 1) + (size_t)(cells / ENT_BLOCK + 1) * 16;
    }
    return b;
}
static_assert(GROUP_FIXED_BYTES >= 16 * GRAIN, "room for rounding every array of a batch");

}  // namespace

struct mesh_server {
    int device = 0;
    char *arena = nullptr;
    Pool pool;
    int max_wave = 256, max_queue = 1 << 20;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<int64_t> queue;
    std::unordered_map<int64_t, Req> reqs;
    int64_t next_id = 1;
    std::vector<Slot> slots;
    std::thread th;
    bool stop = false;
    std::string msg;
    // statistics
    std::vector<double> lat_ms;
    int64_t rejected = 0, failed = 0, waves = 0, wave_reqs = 0;
    double samples = 0;
    bool have_t0 = false;
    clk::time_point t0, t_last;
};

namespace {

int sfail(mesh_server *s, int status, const std::string &m) {
    s->msg = m;
    return status;
}

// Worst-case output of a request (vertices / faces) and its output block size.
void bounds(Req *r) {
    const int64_t nx = r->dims[0], ny = r->dims[1], nz = r->dims[2];
    const bool cells = nx > 1 && ny > 1 && nz > 1;
    const int64_t nc = cells ? (nx - 1) * (ny - 1) * (nz - 1) : 0, nn = cells ? nx * ny * nz : 0;
    switch (r->p.alg) {
    case MESH_ALG_MC:
    case MESH_ALG_MC_WELDED: r->vcap = 12 * nc; r->fcap = 5 * nc; break;
    case MESH_ALG_MT: r->vcap = 7 * nn; r->fcap = 12 * nc; break;
    default: r->vcap = nc; r->fcap = 6 * nn; break;
    }
    r->vbytes = up((size_t)r->vcap * 3 * (r->out64 ? 8 : 4));
}
size_t out_bytes(const Req &r) { return r.vbytes + up((size_t)r.fcap * 24); }
// Pool bytes a request holds while in flight: outputs, and a host volume's copy.
size_t held_bytes(const Req &r) { return out_bytes(r) + (r.host_vol ? up(r.vol_bytes) : 0); }

struct GroupKey {
    int T, iso_type, range_type;
    double iso;
};
bool same_key(const Group &g, const Req &r) {
    return g.T == r.T && g.iso_type == r.p.iso_type && g.range_type == r.p.range_type &&
           memcmp(&g.iso, &r.p.iso, sizeof(double)) == 0;
}

// Takes queued requests into slot `sl` while their outputs and the batches'
// scratch fit the pool.  A wave reserves at most its slot's share of the pool
// (beyond its first request): one wave taking all the memory of a backlog would
// leave the other slots idle and the device running one wave at a time.
// Called with the lock held.
void form_wave(mesh_server *s, Slot &sl) {
    sl.groups.clear();
    sl.singles.clear();
    sl.wave.clear();
    int admitted = 0;
    const size_t share_cap = s->pool.cap / s->slots.size();
    size_t reserved = 0;
    while (!s->queue.empty() && admitted < s->max_wave) {
        Req &r = s->reqs[s->queue.front()];
        const size_t est = held_bytes(r) + (r.p.alg == MESH_ALG_MC ? vol_scratch_bytes(r) : 0);
        if (admitted && reserved + est > share_cap) break;
        reserved += est;
        int gi = -1;
        if (r.p.alg == MESH_ALG_MC) {
            for (size_t g = 0; g < sl.groups.size(); g++)
                if (same_key(sl.groups[g], r)) gi = (int)g;
            if (gi < 0 && (int)sl.groups.size() == MAX_GROUPS) break;
        }
        if (!s->pool.alloc(out_bytes(r), &r.out)) break;
        if (r.host_vol && !s->pool.alloc(up(r.vol_bytes), &r.vin)) {
            s->pool.release(&r.out);
            break;
        }
        if (r.p.alg == MESH_ALG_MC) {
            if (gi < 0) {
                Group g;
                g.T = r.T;
                g.iso_type = r.p.iso_type;
                g.range_type = r.p.range_type;
                g.iso = r.p.iso;
                sl.groups.push_back(g);
                gi = (int)sl.groups.size() - 1;
            }
            Group &grp = sl.groups[gi];
            const size_t share = vol_scratch_bytes(r);
            grp.reqs.push_back(r.id);
            grp.bound += share;
            // the batches' scratch must still fit next to the outputs
            size_t need = 0, largest = 0;
            for (auto &g : sl.groups) {
                need += g.bound;
                largest = std::max(largest, g.bound);
            }
            if (need > s->pool.cap - s->pool.used || largest > s->pool.largest()) {
                grp.reqs.pop_back();
                grp.bound -= share;
                if (grp.reqs.empty()) sl.groups.erase(sl.groups.begin() + gi);
                s->pool.release(&r.out);
                s->pool.release(&r.vin);
                break;
            }
        } else {
            sl.singles.push_back(r.id);
        }
        s->queue.pop_front();
        r.state = RQ_RUNNING;
        sl.wave[r.id] = r;
        admitted++;
    }
    // scratch blocks; if first-fit cannot place one, hand that batch's requests back
    for (size_t g = 0; g < sl.groups.size();) {
        if (s->pool.alloc(sl.groups[g].bound, &sl.groups[g].scratch)) {
            g++;
            continue;
        }
        for (auto it = sl.groups[g].reqs.rbegin(); it != sl.groups[g].reqs.rend(); ++it) {
            Req &r = s->reqs[*it];
            s->pool.release(&r.out);
            s->pool.release(&r.vin);
            r.state = RQ_QUEUED;
            s->queue.push_front(*it);
            sl.wave.erase(*it);
        }
        sl.groups.erase(sl.groups.begin() + g);
    }
}

// Fails the requests of a wave that will not complete, frees its scratch and
// the slot.  Called with the lock held.
void fail_wave(mesh_server *s, Slot &sl, int rc) {
    for (auto &g : sl.groups) {
        for (int64_t id : g.reqs) {
            Req &r = s->reqs[id];
            r.state = RQ_FAILED;
            r.status = rc;
            s->pool.release(&r.vin);
            s->failed++;
        }
        s->pool.release(&g.scratch);
    }
    for (int64_t id : sl.singles) {
        Req &r = s->reqs[id];
        r.state = RQ_FAILED;
        r.status = rc;
        s->pool.release(&r.vin);
        s->failed++;
    }
    sl.groups.clear();
    sl.singles.clear();
    sl.wave.clear();
    sl.finishing = 0;
    sl.busy = 0;
    s->cv.notify_all();
}

// Publishes the results of slot sl's wave and frees the slot.  Lock held.
void complete_wave(mesh_server *s, Slot &sl, clk::time_point now) {
    auto finish = [&](int64_t id) {
        Req &r = s->reqs[id];
        r.t_done = now;
        if (r.status) {
            r.state = RQ_FAILED;
            s->failed++;
            return;
        }
        r.state = RQ_DONE;
        s->lat_ms.push_back(std::chrono::duration<double, std::milli>(now - r.t_sub).count());
        s->samples += (double)r.dims[0] * r.dims[1] * r.dims[2];
        s->t_last = now;
    };
    for (auto &g : sl.groups)
        for (int64_t id : g.reqs) finish(id);
    for (int64_t id : sl.singles) finish(id);
    sl.groups.clear();
    sl.singles.clear();
    sl.wave.clear();
    sl.finishing = 0;
    sl.busy = 0;
    s->cv.notify_all();
}

// Host function queued after a wave's kernels.  Each finished mesh keeps the
// start of its worst-case block and frees the rest, and the wave's scratch is
// freed.  Held meshes left where the worst-case blocks were can split the free
// space into holes too small for the next worst case (the queue's head, or one
// like this wave's): then the loop thread first moves them to the top of the
// pool (finish_wave); otherwise the wave is complete.
void CUDART_CB wave_done(void *arg) {
    WaveTag *tag = (WaveTag *)arg;
    Slot *sl = tag->sl;
    const uint64_t seq = tag->seq;
    delete tag;
    mesh_server *s = sl->srv;
    const clk::time_point now = clk::now();
    std::lock_guard<std::mutex> lk(s->mu);
    if (seq != sl->seq || !sl->busy) return;  // this wave was already failed
    size_t room = 0;  // the largest worst case of the wave
    auto record = [&](Req &r, int64_t nv, int64_t nf, unsigned err) {
        room = std::max(room, r.out.size);
        s->pool.release(&r.vin);  // the wave's kernels are done with a host volume's copy
        if (err) {  // the worst-case block stays reserved until the release
            r.status = (err & ERR_CAPACITY) ? MESH_ECAPACITY : MESH_EDEVICE;
            return;
        }
        r.nverts = nv;
        r.nfaces = nf;
        const size_t vb = up((size_t)nv * 3 * (r.out64 ? 8 : 4)), fb = up((size_t)nf * 24);
        r.keep_v = Block{r.out.off, vb};
        r.keep_f = Block{r.out.off + r.vbytes, fb};
        s->pool.release_range(r.out.off + vb, r.vbytes - vb);
        s->pool.release_range(r.out.off + r.vbytes + fb, r.out.size - r.vbytes - fb);
        r.out.size = 0;
    };
    for (auto &g : sl->groups) {
        const int64_t *o = sl->res + g.res_off;  // offsets [n+1][2], then the error word
        const size_t n = g.reqs.size();
        const unsigned err = (unsigned)(o[2 * (n + 1)] & 0xffffffffll);
        for (size_t i = 0; i < n; i++)
            record(s->reqs[g.reqs[i]], o[2 * i + 2] - o[2 * i], o[2 * i + 3] - o[2 * i + 1], err);
        s->pool.release(&g.scratch);
    }
    for (size_t i = 0; i < sl->singles.size(); i++) {
        const int64_t *o = sl->res + sl->single_res_off + 3 * i;
        record(s->reqs[sl->singles[i]], o[0], o[1], (unsigned)(o[2] & 0xffffffffll));
    }
    if (!s->queue.empty()) {
        const Req &h = s->reqs[s->queue.front()];
        room = std::max(room, held_bytes(h) + (h.p.alg == MESH_ALG_MC ? vol_scratch_bytes(h) : 0));
    }
    if (s->pool.largest() < room) {
        sl->finishing = 1;
        s->cv.notify_all();
        return;
    }
    complete_wave(s, *sl, now);
}

// Host function queued after the mesh moves: the meshes are in their new
// blocks, the old ones are freed and the wave is complete.
void CUDART_CB moves_done(void *arg) {
    WaveTag *tag = (WaveTag *)arg;
    Slot *sl = tag->sl;
    const uint64_t seq = tag->seq;
    delete tag;
    mesh_server *s = sl->srv;
    const clk::time_point now = clk::now();
    std::lock_guard<std::mutex> lk(s->mu);
    if (seq != sl->seq || !sl->busy) return;
    auto settle = [&](int64_t id) {
        Req &r = s->reqs[id];
        if (!r.move_v.size && !r.move_f.size) return;
        s->pool.release(&r.keep_v);
        s->pool.release(&r.keep_f);
        r.keep_v = r.move_v;
        r.keep_f = r.move_f;
        r.move_v.size = r.move_f.size = 0;
    };
    for (auto &g : sl->groups)
        for (int64_t id : g.reqs) settle(id);
    for (int64_t id : sl->singles) settle(id);
    complete_wave(s, *sl, now);
}

// Moves every finished mesh of slot sl into blocks at the top of the pool
// (leaving a mesh in place when they do not fit), then queues moves_done.
// Called with the lock held; unlocks around the CUDA calls.
void finish_wave(mesh_server *s, Slot &sl, std::unique_lock<std::mutex> &lk) {
    sl.finishing = 0;
    struct Move {
        size_t src, dst, bytes;
    };
    std::vector<Move> moves;
    auto plan = [&](int64_t id) {
        Req &r = s->reqs[id];
        const size_t vb = r.keep_v.size, fb = r.keep_f.size;
        if (r.status || (!vb && !fb)) return;
        Block bv, bf;
        if (vb && !s->pool.alloc_top(vb, &bv)) return;
        if (fb && !s->pool.alloc_top(fb, &bf)) {
            s->pool.release(&bv);
            return;
        }
        if (vb) moves.push_back({r.keep_v.off, bv.off, vb});
        if (fb) moves.push_back({r.keep_f.off, bf.off, fb});
        r.move_v = bv;
        r.move_f = bf;
    };
    for (auto &g : sl.groups)
        for (int64_t id : g.reqs) plan(id);
    for (int64_t id : sl.singles) plan(id);
    const uint64_t seq = sl.seq;
    lk.unlock();
    cudaError_t e = cudaSuccess;
    for (const Move &m : moves)
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(s->arena + m.dst, s->arena + m.src, m.bytes, cudaMemcpyDeviceToDevice, sl.stream);
    WaveTag *tag = nullptr;
    if (e == cudaSuccess) {
        tag = new (std::nothrow) WaveTag{&sl, seq};
        e = tag ? cudaLaunchHostFunc(sl.stream, moves_done, tag) : cudaErrorMemoryAllocation;
        if (e != cudaSuccess) delete tag;
    }
    lk.lock();
    if (e != cudaSuccess) {
        s->msg = std::string("moving finished meshes: ") + cudaGetErrorString(e);
        fail_wave(s, sl, MESH_ECUDA);
    }
}

cudaError_t ensure_pinned(void **p, size_t *cap, size_t n) {
    if (n <= *cap) return cudaSuccess;
    const size_t want = std::max(n, 2 * *cap);
    if (*p) cudaFreeHost(*p);
    *p = nullptr;
    *cap = 0;
    cudaError_t e = cudaHostAlloc(p, want, cudaHostAllocDefault);
    if (e == cudaSuccess) *cap = want;
    return e;
}

// Queues a formed wave on the slot's stream (no lock held; the wave's
// requests are owned by the slot until wave_done).
int launch_wave(mesh_server *s, Slot &sl) {
    cudaError_t e;
    // pinned results: per batch (n+1)*2 offsets + error word; 3 words per single request
    size_t words = 0;
    for (auto &g : sl.groups) {
        g.res_off = words;
        words += 2 * (g.reqs.size() + 1) + 1;
    }
    sl.single_res_off = words;
    words += 3 * sl.singles.size();
    {
        void *p = sl.res;
        size_t cap = sl.res_cap * 8;
        if ((e = ensure_pinned(&p, &cap, words * 8 + 8)) != cudaSuccess) return MESH_ENOMEM;
        sl.res = (int64_t *)p;
        sl.res_cap = cap / 8;
        memset(sl.res, 0, words * 8 + 8);  // error words are copied into their low halves
    }
    // host volumes go up first, into their pool blocks; the wave reads those
    for (auto &kv : sl.wave) {
        Req &r = kv.second;
        if (!r.host_vol) continue;
        if (r.vol_bytes &&
            (e = cudaMemcpyAsync(s->arena + r.vin.off, r.host_vol, r.vol_bytes, cudaMemcpyHostToDevice, sl.stream)) !=
                cudaSuccess)
            return MESH_ECUDA;
        r.vol = s->arena + r.vin.off;
    }
    // exact layouts; every batch gets its own region of the pinned staging
    std::vector<GroupLayout> lays(sl.groups.size());
    size_t stage = 0;
    for (size_t gi = 0; gi < sl.groups.size(); gi++) {
        std::vector<const Req *> rs;
        for (int64_t id : sl.groups[gi].reqs) rs.push_back(&sl.wave.at(id));
        layout_group(rs, &lays[gi]);
        if (lays[gi].z.items >= ((int64_t)1 << 31) / WY) return MESH_ETOOLARGE;  // 32-bit compaction counter
        if (lays[gi].total > sl.groups[gi].scratch.size) return MESH_EDEVICE;  // bound violated: never launch
        sl.groups[gi].stage_off = stage;
        stage += up(lays[gi].head);
    }
    {
        void *st = sl.stage;
        if ((e = ensure_pinned(&st, &sl.stage_cap, stage + 8)) != cudaSuccess) return MESH_ENOMEM;
        sl.stage = (char *)st;
    }
    for (size_t gi = 0; gi < sl.groups.size(); gi++) {
        Group &g = sl.groups[gi];
        GroupLayout &L = lays[gi];
        std::vector<const Req *> rs;
        for (int64_t id : g.reqs) rs.push_back(&sl.wave.at(id));
        char *blk = s->arena + g.scratch.off;
        const int n = (int)rs.size();
        Plan P{};
        mesh_params prm = rs[0]->p;
        int Q64 = 0, A64 = 0, P64 = 0;
        set_types(P, g.T, &prm, &Q64, &A64, &P64);
        const int L32 = prm.range_type == MESH_DT_F32;
        std::vector<uint32_t> ivol, svol;
        batch_owners(L.hv, L.z, ivol, svol);
        std::vector<TabJob> jobs;
        for (int v = 0; v < n; v++) {
            BatchVol &bv = L.hv[v];
            const Req &r = *rs[v];
            bv.vol = r.vol;
            bv.tabs = (const double *)(blk + L.o_tabs) + L.tab_off[v];
            bv.verts = s->arena + r.out.off;
            bv.faces = (int64_t *)(s->arena + r.out.off + r.vbytes);
            bv.vcap = r.vcap;
            bv.fcap = r.fcap;
            if (!bv.cx) continue;
            TabJob j;
            j.dst = (double *)(blk + L.o_tabs) + L.tab_off[v];
            j.nx = bv.nx; j.ny = bv.ny; j.nz = bv.nz;
            memcpy(j.range, r.p.range, sizeof(j.range));
            jobs.push_back(j);
        }
        // head: descriptors, owners, table jobs -- one copy from pinned staging
        char *hs = sl.stage + g.stage_off;
        memcpy(hs, L.hv.data(), sizeof(BatchVol) * n);
        if (!ivol.empty()) memcpy(hs + L.o_ivol, ivol.data(), 4 * ivol.size());
        if (!svol.empty()) memcpy(hs + L.o_svol, svol.data(), 4 * svol.size());
        if (!jobs.empty()) memcpy(hs + L.o_jobs, jobs.data(), sizeof(TabJob) * jobs.size());
        if ((e = cudaMemcpyAsync(blk, hs, L.head, cudaMemcpyHostToDevice, sl.stream)) != cudaSuccess)
            return MESH_ECUDA;
        if (!jobs.empty() &&
            (e = launch_tables_batch((const TabJob *)(blk + L.o_jobs), (int)jobs.size(), L.z.max_ntab, L32,
                                     sl.stream)) != cudaSuccess)
            return MESH_ECUDA;
        P.pstride = L.z.pieces;
        P.cnt = (uint32_t *)(blk + L.o_cnt);
        P.base = (int64_t *)(blk + L.o_base);
        P.flags = (uint8_t *)(blk + L.o_flags);
        P.scan_state = (unsigned long long *)(blk + L.o_scan);
        P.scan_ticket = (unsigned int *)(blk + L.o_scan + (size_t)std::max<int64_t>(L.z.stiles, n) * NCNT * 8);
        P.totals = (int64_t *)(blk + L.o_misc);
        P.err = (unsigned int *)((int64_t *)(blk + L.o_misc) + NCNT);
        P.work = (unsigned int *)((int64_t *)(blk + L.o_misc) + NCNT + 1);
        P.scan_spin_limit = 1 << 24;
        P.bvols = (const BatchVol *)blk;
        P.item_vol = (const uint32_t *)(blk + L.o_ivol);
        P.stile_vol = (const uint32_t *)(blk + L.o_svol);
        P.vol_off = (int64_t *)(blk + L.o_offs);
        P.nitems = L.z.items;
        P.nvols = n;
        P.nstiles = (int32_t)L.z.stiles;
        P.vol_outputs = 1;
        P.ent_pos = (unsigned long long *)(blk + L.o_pos);
        P.ent_val = blk + L.o_val;
        P.ent_side = (long long *)(blk + L.o_side);
        P.ent_vol = (uint32_t *)(blk + L.o_vol);
        P.ent_cs = (uint8_t *)(blk + L.o_cs);
        P.ent_cap = L.cells;
        P.verts_cap = P.faces_cap = (int64_t)1 << 62;  // each volume checks its own block
        if ((e = cudaMemsetAsync(blk + L.o_misc, 0, MISC_SLOTS * 8, sl.stream)) != cudaSuccess ||
            (e = launch_classify_batch(P, 0, sl.stream)) != cudaSuccess ||
            (e = launch_scan_batch(P, L.scan_vol ? 1024 : 256, sl.stream, L.scan_vol)) != cudaSuccess ||
            (e = launch_compact_batch(P, 0, sl.stream)) != cudaSuccess ||
            (e = launch_expand_batch(P, Q64, P64, sl.stream)) != cudaSuccess ||
            (e = cudaMemcpyAsync(sl.res + g.res_off, P.vol_off, 16 * (size_t)(n + 1), cudaMemcpyDeviceToHost,
                                 sl.stream)) != cudaSuccess ||
            (e = cudaMemcpyAsync(sl.res + g.res_off + 2 * (n + 1), P.err, 4, cudaMemcpyDeviceToHost, sl.stream)) !=
                cudaSuccess)
            return MESH_ECUDA;
    }
    if (!sl.singles.empty()) {
        const size_t need = 3 * sl.singles.size() * 8;
        if (need > sl.d_counts_cap) {
            if (sl.d_counts) cudaFree(sl.d_counts);
            sl.d_counts = nullptr;
            sl.d_counts_cap = 0;
            if ((e = cudaMalloc((void **)&sl.d_counts, 2 * need)) != cudaSuccess) return MESH_ENOMEM;
            sl.d_counts_cap = 2 * need;
        }
        if ((e = cudaMemsetAsync(sl.d_counts, 0, need, sl.stream)) != cudaSuccess) return MESH_ECUDA;
        for (size_t i = 0; i < sl.singles.size(); i++) {
            const Req &r = sl.wave.at(sl.singles[i]);
            if (r.p.alg == MESH_ALG_MC_WELDED) {
                // the context's welded extraction (it waits for the slot's stream),
                // then a device copy of the welded mesh into the output block
                int64_t cnt[3] = {0, 0, 0};
                int rc = mesh_count(sl.ctx, r.vol, r.T, r.dims[0], r.dims[1], r.dims[2], 1, &r.p, &cnt[0], &cnt[1]);
                if (rc == MESH_OK && (cnt[0] > r.vcap || cnt[1] > r.fcap)) rc = MESH_ECAPACITY;
                if (rc == MESH_OK)
                    rc = mesh_fill(sl.ctx, s->arena + r.out.off, (int64_t *)(s->arena + r.out.off + r.vbytes), 1);
                if (rc) return rc;
                // (a pageable source: the copy takes the values before it returns)
                if ((e = cudaMemcpyAsync(sl.d_counts + 3 * i, cnt, sizeof(cnt), cudaMemcpyHostToDevice, sl.stream)) !=
                    cudaSuccess)
                    return MESH_ECUDA;
                continue;
            }
            int rc = mesh_extract_device(sl.ctx, r.vol, r.T, r.dims[0], r.dims[1], r.dims[2], &r.p,
                                         s->arena + r.out.off, r.vcap, (int64_t *)(s->arena + r.out.off + r.vbytes),
                                         r.fcap, sl.d_counts + 3 * i);
            if (rc) return rc;
            // the context's error word of this request
            if (sl.ctx->plan.err &&
                (e = cudaMemcpyAsync(sl.d_counts + 3 * i + 2, sl.ctx->plan.err, 4, cudaMemcpyDeviceToDevice,
                                     sl.stream)) != cudaSuccess)
                return MESH_ECUDA;
        }
        if ((e = cudaMemcpyAsync(sl.res + sl.single_res_off, sl.d_counts, need, cudaMemcpyDeviceToHost, sl.stream)) !=
            cudaSuccess)
            return MESH_ECUDA;
    }
    WaveTag *tag = new (std::nothrow) WaveTag{&sl, sl.seq};
    if (!tag) return MESH_ENOMEM;
    e = cudaLaunchHostFunc(sl.stream, wave_done, tag);
    if (e != cudaSuccess) delete tag;
    return e == cudaSuccess ? MESH_OK : MESH_ECUDA;
}

void loop(mesh_server *s) {
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        auto free_slot = [&]() {
            for (auto &sl : s->slots)
                if (!sl.busy) return &sl;
            return (Slot *)nullptr;
        };
        // a wave whose stream reports an error never reaches wave_done: fail it
        auto reap = [&]() {
            for (auto &sl : s->slots) {
                if (!sl.busy || sl.launching) continue;
                const cudaError_t e = cudaStreamQuery(sl.stream);
                if (e != cudaSuccess && e != cudaErrorNotReady) {
                    s->msg = std::string("wave failed on the device: ") + cudaGetErrorString(e);
                    fail_wave(s, sl, MESH_ECUDA);
                }
            }
        };
        auto finishing = [&]() {
            for (auto &sl : s->slots)
                if (sl.busy && sl.finishing) return &sl;
            return (Slot *)nullptr;
        };
        while (!s->cv.wait_for(lk, std::chrono::milliseconds(50),
                               [&] { return s->stop || finishing() || (!s->queue.empty() && free_slot()); }))
            reap();
        if (s->stop) break;
        if (Slot *fs = finishing()) {
            finish_wave(s, *fs, lk);
            continue;
        }
        Slot &sl = *free_slot();
        form_wave(s, sl);
        if (sl.groups.empty() && sl.singles.empty()) {
            // the head does not fit now: wait for a wave to finish or a release
            s->cv.wait_for(lk, std::chrono::milliseconds(50));
            reap();
            continue;
        }
        sl.busy = 1;
        sl.launching = 1;
        sl.seq++;
        s->waves++;
        for (auto &g : sl.groups) s->wave_reqs += (int64_t)g.reqs.size();
        s->wave_reqs += (int64_t)sl.singles.size();
        lk.unlock();
        const int rc = launch_wave(s, sl);
        lk.lock();
        sl.launching = 0;
        if (rc) {  // nothing of this wave will complete: fail its requests
            s->msg = "wave launch failed";
            lk.unlock();
            cudaStreamSynchronize(sl.stream);
            lk.lock();
            fail_wave(s, sl, rc);
        }
    }
}

void fill_result(const mesh_server *s, const Req &r, int *state, int64_t *nv, int64_t *nf, void **v, int64_t **f) {
    if (state) *state = r.state;
    if (nv) *nv = r.state == RQ_DONE ? r.nverts : 0;
    if (nf) *nf = r.state == RQ_DONE ? r.nfaces : 0;
    if (v) *v = r.state == RQ_DONE ? (void *)(s->arena + r.keep_v.off) : nullptr;
    if (f) *f = r.state == RQ_DONE ? (int64_t *)(s->arena + r.keep_f.off) : nullptr;
}

}  // namespace

extern "C" {

int mesh_server_create(int device, int64_t budget_bytes, int slots, int max_wave, int max_queue, mesh_server **out) {
    if (!out || budget_bytes <= 0 || slots < 1 || slots > 16 || max_wave < 1 || max_queue < 1) return MESH_EINVAL;
    *out = nullptr;
    if (cudaSetDevice(device) != cudaSuccess) return MESH_ECUDA;
    mesh_server *s = new (std::nothrow) mesh_server();
    if (!s) return MESH_ENOMEM;
    s->device = device;
    s->max_wave = max_wave;
    s->max_queue = max_queue;
    if (cudaMalloc((void **)&s->arena, (size_t)budget_bytes) != cudaSuccess) {
        cudaGetLastError();
        delete s;
        return MESH_ENOMEM;
    }
    s->pool.init((size_t)budget_bytes);
    s->slots.resize(slots);
    for (int i = 0; i < slots; i++) {
        Slot &sl = s->slots[i];
        sl.srv = s;
        sl.index = i;
        if (cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) != cudaSuccess ||
            mesh_ctx_create(device, &sl.ctx) != MESH_OK) {
            cudaGetLastError();
            mesh_server_destroy(s);
            return MESH_ENOMEM;
        }
        mesh_ctx_set_stream(sl.ctx, sl.stream);
    }
    s->th = std::thread(loop, s);
    *out = s;
    return MESH_OK;
}

void mesh_server_destroy(mesh_server *s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->cv.notify_all();
    }
    if (s->th.joinable()) s->th.join();
    cudaSetDevice(s->device);
    for (auto &sl : s->slots) {
        if (sl.stream) cudaStreamSynchronize(sl.stream);  // runs the last wave_done
        if (sl.ctx) mesh_ctx_destroy(sl.ctx);
        if (sl.stream) cudaStreamDestroy(sl.stream);
        if (sl.stage) cudaFreeHost(sl.stage);
        if (sl.res) cudaFreeHost(sl.res);
        if (sl.d_counts) cudaFree(sl.d_counts);
    }
    if (s->arena) cudaFree(s->arena);
    delete s;
}

const char *mesh_server_last_error(const mesh_server *s) { return s ? s->msg.c_str() : ""; }

int mesh_server_submit(mesh_server *s, const void *vol, int vol_dtype, int64_t nx, int64_t ny, int64_t nz,
                       int vol_on_device, const mesh_params *p, int64_t *id) {
    if (!s || !p || !id) return MESH_EINVAL;
    *id = 0;
    int rc = validate(nullptr, vol_dtype, nx, ny, nz, p);
    if (rc) return sfail(s, rc, "invalid request");
    if (!vol && nx > 1 && ny > 1 && nz > 1) return sfail(s, MESH_EINVAL, "volume is NULL");
    Req r;
    if (vol_on_device) {
        r.vol = vol;
    } else if (nx > 1 && ny > 1 && nz > 1) {
        r.host_vol = vol;
        r.vol_bytes = (size_t)nx * ny * nz * dtype_size(vol_dtype);
    }
    r.T = vol_dtype;
    r.dims[0] = nx; r.dims[1] = ny; r.dims[2] = nz;
    r.p = *p;
    int bits = 32;
    mesh_output_float_bits(vol_dtype, p, &bits);
    r.out64 = bits == 64;
    bounds(&r);
    std::lock_guard<std::mutex> lk(s->mu);
    if (!s->have_t0) {
        s->have_t0 = true;
        s->t0 = clk::now();
    }
    // the worst case alone (with its batch scratch and a host volume's copy) must fit the whole pool
    size_t need = held_bytes(r);
    if (r.p.alg == MESH_ALG_MC) need += GROUP_FIXED_BYTES + vol_scratch_bytes(r);
    if (need > s->pool.cap) {
        s->rejected++;
        return sfail(s, MESH_EBUDGET, "request's worst case exceeds the memory budget");
    }
    if ((int64_t)s->queue.size() >= s->max_queue) {
        s->rejected++;
        return sfail(s, MESH_EBUSY, "queue full");
    }
    r.id = s->next_id++;
    r.t_sub = clk::now();
    *id = r.id;
    s->reqs.emplace(r.id, r);
    s->queue.push_back(r.id);
    s->cv.notify_all();
    return MESH_OK;
}

int mesh_server_poll(mesh_server *s, int64_t id, int *state, int64_t *nverts, int64_t *nfaces, void **verts,
                     int64_t **faces) {
    if (!s) return MESH_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return sfail(s, MESH_EINVAL, "unknown request");
    fill_result(s, it->second, state, nverts, nfaces, verts, faces);
    return it->second.state == RQ_FAILED ? it->second.status : MESH_OK;
}

int mesh_server_wait(mesh_server *s, int64_t id, int64_t timeout_us, int *state, int64_t *nverts, int64_t *nfaces,
                     void **verts, int64_t **faces) {
    if (!s) return MESH_EINVAL;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return sfail(s, MESH_EINVAL, "unknown request");
    s->cv.wait_for(lk, std::chrono::microseconds(timeout_us), [&] {
        const int st = s->reqs[id].state;
        return st == RQ_DONE || st == RQ_FAILED;
    });
    const Req &r = s->reqs[id];
    fill_result(s, r, state, nverts, nfaces, verts, faces);
    return r.state == RQ_FAILED ? r.status : MESH_OK;
}

int mesh_server_release(mesh_server *s, int64_t id) {
    if (!s) return MESH_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return sfail(s, MESH_EINVAL, "unknown request");
    if (it->second.state == RQ_QUEUED || it->second.state == RQ_RUNNING)
        return sfail(s, MESH_ESTATE, "request still in flight");
    for (Block *b : {&it->second.out, &it->second.keep_v, &it->second.keep_f, &it->second.move_v,
                     &it->second.move_f, &it->second.vin})
        s->pool.release(b);
    s->reqs.erase(it);
    s->cv.notify_all();
    return MESH_OK;
}

int mesh_server_stats(mesh_server *s, double *st) {
    if (!s || !st) return MESH_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    std::vector<double> l = s->lat_ms;
    std::sort(l.begin(), l.end());
    auto pct = [&](double q) { return l.empty() ? 0.0 : l[std::min(l.size() - 1, (size_t)(q * (l.size() - 1) + 0.5))]; };
    double mean = 0;
    for (double x : l) mean += x;
    const double wall = s->have_t0 ? std::chrono::duration<double>(s->t_last - s->t0).count() : 0;
    st[0] = (double)l.size();
    st[1] = (double)s->rejected;
    st[2] = (double)s->failed;
    st[3] = pct(0.5);
    st[4] = pct(0.99);
    st[5] = l.empty() ? 0 : mean / l.size();
    st[6] = s->samples;
    st[7] = wall;
    st[8] = (double)s->pool.peak;
    st[9] = (double)s->pool.cap;
    st[10] = (double)s->queue.size();
    st[11] = (double)s->pool.used;
    st[12] = (double)s->waves;
    st[13] = s->waves ? (double)s->wave_reqs / s->waves : 0;
    return MESH_OK;
}

int mesh_server_replay(mesh_server *s, int n, const void *const *vols, const int *dtypes, const int64_t *dims,
                       const mesh_params *params, const double *arrivals_s) {
    if (!s || n < 0 || (n && (!vols || !dtypes || !dims || !params || !arrivals_s))) return MESH_EINVAL;
    std::vector<int64_t> ids;
    std::mutex m;
    std::condition_variable cv;
    bool done_submitting = false, stuck = false;
    // releaser: frees every request as soon as it ends, in submission order
    std::thread rel([&] {
        size_t k = 0;
        for (;;) {
            int64_t id;
            {
                std::unique_lock<std::mutex> lk(m);
                cv.wait(lk, [&] { return k < ids.size() || done_submitting; });
                if (k == ids.size()) return;
                id = ids[k++];
            }
            if (id <= 0) continue;
            int st = 0, tries = 0;
            // a request that has not ended after 120 s is reported, not waited for
            while (mesh_server_wait(s, id, 1000000, &st, nullptr, nullptr, nullptr, nullptr) == MESH_OK &&
                   st != RQ_DONE && ++tries < 120)
                ;
            if (st == RQ_QUEUED || st == RQ_RUNNING) {
                std::lock_guard<std::mutex> lk(m);
                stuck = true;
                continue;
            }
            mesh_server_release(s, id);
        }
    });
    const clk::time_point t0 = clk::now();
    for (int i = 0; i < n; i++) {
        const clk::time_point due = t0 + std::chrono::duration_cast<clk::duration>(
                                              std::chrono::duration<double>(arrivals_s[i]));
        for (;;) {  // sleep through long gaps, spin through short ones
            const auto left = due - clk::now();
            if (left <= clk::duration::zero()) break;
            if (left > std::chrono::microseconds(300)) std::this_thread::sleep_for(left - std::chrono::microseconds(200));
        }
        int64_t id = 0;
        const int rc = mesh_server_submit(s, vols[i], dtypes[i], dims[3 * i], dims[3 * i + 1], dims[3 * i + 2], 1,
                                          &params[i], &id);
        std::lock_guard<std::mutex> lk(m);
        ids.push_back(rc == MESH_OK ? id : -1);
        cv.notify_all();
    }
    {
        std::lock_guard<std::mutex> lk(m);
        done_submitting = true;
        cv.notify_all();
    }
    rel.join();
    return stuck ? sfail(s, MESH_EDEVICE, "a replayed request did not end within 120 s") : MESH_OK;
}

int mesh_server_reset_stats(mesh_server *s) {
    if (!s) return MESH_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    s->lat_ms.clear();
    s->rejected = s->failed = s->waves = s->wave_reqs = 0;
    s->samples = 0;
    s->have_t0 = false;
    s->pool.peak = s->pool.used;
    return MESH_OK;
}

}  // extern "C"
