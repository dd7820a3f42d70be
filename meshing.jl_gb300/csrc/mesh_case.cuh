// Marching Cubes case words in the index order of the ballot walks
// (k_classify.cu, k_emit_mc.cu).
//
// A walk lane holds, per sample row, the 2-bit field (x, x+1) of `v < iso`
// bits.  Index bits 0..7 are the corners (x,y,z) (x+1,y,z) (x,y,z+1)
// (x+1,y,z+1) (x,y+1,z) (x+1,y+1,z) (x,y+1,z+1) (x+1,y+1,z+1): the lane's
// fields of row y in planes z and z+1, then of row y+1.  The cube case of
// src/common.jl:10-20 (corner order of src/marching_cubes.jl:42-49) is a
// permutation of these bits.  Include after mesh_tables.h.
#pragma once

namespace mesh {
namespace {

// Packed word of a case: vertices (bits 0-11), faces (bits 12-22) and, for an
// active cell (case not 0x00 / 0xff), 1 << 23.  Sums of at most ZC such words
// do not carry between fields.
constexpr uint32_t PK_F = 12, PK_A = 23;
static_assert(12 * ZC < (1 << PK_F) && 5 * ZC < (1 << (PK_A - PK_F)) && ZC < (1 << (32 - PK_A)),
              "packed chunk counts must not carry into the next field");

__device__ __forceinline__ unsigned mc_case_of_index(unsigned u) {
    return (u & 1u) | (((u >> 1) & 1u) << 1) | (((u >> 5) & 1u) << 2) | (((u >> 4) & 1u) << 3) |
           (((u >> 2) & 1u) << 4) | (((u >> 3) & 1u) << 5) | (((u >> 7) & 1u) << 6) | (((u >> 6) & 1u) << 7);
}

// s_pk[i]: packed word of index i; s_case[i] (if given): its cube case.
__device__ __forceinline__ void load_tables_mc_packed(uint32_t *s_pk, uint8_t *s_case = nullptr) {
    for (int i = threadIdx.x; i < 256; i += blockDim.x) {
        const unsigned cm = mc_case_of_index((unsigned)i);
        const uint64_t t = MC_CASE_VERTS[cm];
        s_pk[i] = (uint32_t)((t >> 48) & 15u) | ((uint32_t)((t >> 52) & 7u) << PK_F) |
                  ((cm != 0u && cm != 255u) ? (1u << PK_A) : 0u);
        if (s_case) s_case[i] = (uint8_t)cm;
    }
}

// The lane's 4-bit field of one sample row: (x, x+1) in plane z, then in z+1.
__device__ __forceinline__ uint32_t row_field(uint32_t mlo, uint32_t mhi, int lane) {
    return ((mlo >> lane) & 3u) | (((mhi >> lane) & 3u) << 2);
}

// Whether warp tile (tx, ty) of z segment seg lies inside the volume (all 32
// lanes' samples and all WY + 1 sample rows exist) with a segment of fewer
// than 2^32 samples: the walks then take their guard-free form.
__device__ __forceinline__ bool tile_inner(const Plan &p, int tx, int ty, int seg) {
    const int zbeg = seg * p.zs;
    const int zend = min(zbeg + p.zs, p.cz);
    return (int64_t)tx * TILE_X + 32 <= p.nx && (int64_t)ty * WY + WY <= p.cy &&
           (int64_t)(zend - zbeg + 1) * p.nx * p.ny <= (int64_t)0xffffffffu;
}

}  // namespace
}  // namespace mesh
