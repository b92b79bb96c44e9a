// kernels_reuse.cu — the FP32-mixed step with neighbour reuse: candidate
// lists kept between grid builds, the density gather over them (which writes
// the step's neighbour list) and the force gather over that list with the
// whole step fused in. 2D and 3D, summation and continuity density.
//
// A particle's candidate list holds the particles within cutoff + skin of it
// when the grid was last built; while no particle has moved more than skin/2
// since then, every pair within the cutoff is in the lists, and each step
// tests the list instead of the 3^dim stencil cells (the pair set is the
// reference's: the same cutoff test). Each particle's build cell stays its
// reference cell for the cell-relative offsets until the next build.
#include "mixed_common.cuh"
#include "step_particle.cuh"

namespace rrsph {

namespace {

constexpr int kVlBatch = 4;       // list entries the density gather loads together (one uint4)
// neighbours the force gather loads together: four for the 2D common method
// set, two elsewhere (four would spill the registers of the general pair)
template <int DIM, bool STD>
constexpr int kVlForceBatch = DIM == 2 && STD ? 4 : 2;

// List entry = sorted index | cell code << Vl<DIM>::shift, with the code of
// the candidate's cell offset (dx, dy[, dz]) in [-2, 2]^dim:
// (dx + 2) * 5 + (dy + 2) in 2D, ((dx + 2) * 5 + (dy + 2)) * 5 + (dz + 2) in 3D.
template <int DIM>
struct Vl {
    static constexpr int cap = DIM == 3 ? kVerletCap3 : kVerletCap2;
    static constexpr int shift = DIM == 3 ? 25 : 27;
    static constexpr uint32_t index = (1u << shift) - 1u;
    static constexpr uint32_t cmax = DIM == 3 ? 0x3FFu : kMaxCellCoord2;  // largest cell coordinate of a key
};

template <int DIM>
__device__ __forceinline__ uint32_t vl_code(int dx, int dy, int dz) {
    const int c = DIM == 3 ? ((dx + 2) * 5 + (dy + 2)) * 5 + (dz + 2) : (dx + 2) * 5 + (dy + 2);
    return (uint32_t)c << Vl<DIM>::shift;
}
// The offset of an entry's code, shifted by +2 per axis (0..4).
template <int DIM>
__device__ __forceinline__ void vl_offset(uint32_t en, uint32_t& cx, uint32_t& cy, uint32_t& cz) {
    const uint32_t c = en >> Vl<DIM>::shift;
    if (DIM == 3) {
        cx = c / 25u;
        const uint32_t r = c - 25u * cx;
        cy = r / 5u;
        cz = r - 5u * cy;
    } else {
        cx = (c * 13u) >> 6;  // c / 5, exact for c < 32
        cy = c - 5u * cx;
        cz = 0;
    }
}

// The cubic W(q) of kernel_wf as selects: every lane runs the same instructions.
__device__ __forceinline__ float cubic_wf_sel(float f, float q) {
    const float t = 2.0f - q;
    const float w1 = f * ((2.0f / 3.0f - q * q) + q * q * q * 0.5f);
    const float w2 = f * ((1.0f / 6.0f) * (t * t * t));
    return q <= 1.0f ? w1 : (q <= 2.0f ? w2 : 0.0f);
}

__global__ void k_vl_decide(cudaGraphConditionalHandle h, const uint32_t* __restrict__ rebuild) {
    cudaGraphSetConditional(h, *rebuild ? 1u : 0u);
}
__global__ void k_vl_reset(uint32_t* __restrict__ rebuild, uint32_t* __restrict__ gone,
                           unsigned long long* __restrict__ builds) {
    *rebuild = 0u;
    *gone = 0u;
    *builds += 1ull;
}
// After an upload: a flag raised by the key pass that ran for the replaced
// positions is dropped (the next key pass checks the uploaded ones), unless no
// list exists yet (all bits set) or the last build left out a non-existent
// particle or overflowed a list.
__global__ void k_vl_upload_check(uint32_t* __restrict__ rebuild, const uint32_t* __restrict__ gone) {
    if (*rebuild != 0xFFFFFFFFu) *rebuild = *gone ? 1u : 0u;
}

// The window of cell offsets along one axis a particle at offset p from its
// cell's lower edge searches: the cell equals the cutoff and the skin is at
// most h, so a candidate within cutoff + skin lies at most two cells away, and
// two only on the side whose edge is within one skin.
template <int DIM>
__device__ __forceinline__ void vl_window(float p, uint32_t c, float cell, float edge, int& lo, int& hi) {
    lo = (p < edge && c >= 2) ? -2 : (c >= 1 ? -1 : 0);
    hi = (p > cell - edge && c + 2 <= Vl<DIM>::cmax) ? 2 : (c + 1 <= Vl<DIM>::cmax ? 1 : 0);
}

// Distance along one axis from a particle at offset p in [0, cell] from its
// cell's lower edge to the nearest side of the cell d cells away.
__device__ __forceinline__ float gap_to_cell(int d, float p, float cell) {
    return d > 0 ? (float)d * cell - p : (d < 0 ? p - (float)(d + 1) * cell : 0.0f);
}

// After this step's grid (sort + reorder): each particle's candidates, four
// entries gathered in registers and stored as one uint4 into the group's slab
// (the lanes of a warp store neighbouring uint4s), in cell order x outer.
template <int DIM>
__global__ void __launch_bounds__(kMaxGatherThreads) k_vl_build(DevParams P, State S, Sorted G) {
    constexpr int CAP = Vl<DIM>::cap;
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P.n) return;
    const MixedF& M = P.mf;
    const uint32_t id = G.id[k], key = G.key[k];
    const float4 pj = G.P4[k];
    uint32_t cx, cy, cz = 0;
    if (DIM == 3) {
        cx = third_bits(key);
        cy = third_bits(key >> 1);
        cz = third_bits(key >> 2);
        S.bcxy[id] = cx | (cy << 10) | (cz << 20);
        S.boff4[id] = make_float4(pj.x, pj.y, pj.z, 0.0f);
    } else {
        cx = second_bits(key);
        cy = second_bits(key >> 1);
        S.bcxy[id] = cx | (cy << 16);
        S.boff[id] = make_float2(pj.x, pj.y);
    }
    S.slot[id] = k;
    uint4* const slab = reinterpret_cast<uint4*>(G.vlist) + k;  // group g at slab[g * n]
    uint4 buf = make_uint4(kVlNone, kVlNone, kVlNone, kVlNone);
    uint32_t nl = 0;
    if (__float_as_int(pj.w) == P.type_non_existent) atomicOr(S.vl_gone, 1u);
    if (__float_as_int(pj.w) != P.type_non_existent) {
        const float edge = P.vl_skin_edge;
        int x0, x1, y0, y1, z0 = 0, z1 = 0;
        vl_window<DIM>(pj.x, cx, M.cell, edge, x0, x1);
        vl_window<DIM>(pj.y, cy, M.cell, edge, y0, y1);
        if (DIM == 3) vl_window<DIM>(pj.z, cz, M.cell, edge, z0, z1);
#pragma unroll 1
        for (int dx = x0; dx <= x1; dx++) {
#pragma unroll 1
            for (int dy = y0; dy <= y1; dy++) {
#pragma unroll 1
                for (int dz = z0; dz <= z1; dz++) {
                    // a cell none of whose points lies within the list cutoff of the
                    // particle holds no candidate: the distance from the particle
                    // to the cell's nearest side, per axis (the window's corner and
                    // far diagonal cells mostly)
                    const float gx = gap_to_cell(dx, pj.x, M.cell), gy = gap_to_cell(dy, pj.y, M.cell);
                    const float gz = DIM == 3 ? gap_to_cell(dz, pj.z, M.cell) : 0.0f;
                    if (gx * gx + gy * gy + gz * gz >= P.vl_cut2) continue;
                    const uint32_t cell = DIM == 3 ? split3_32(cx + dx) | (split3_32(cy + dy) << 1) |
                                                         (split3_32(cz + dz) << 2)
                                                   : split2_32(cx + dx) | (split2_32(cy + dy) << 1);
                    if (cell >= P.max_cells) continue;
                    const uint32_t s = G.cell_start[cell];
                    if (s == kEmpty) continue;
                    const uint32_t e = G.cell_end[cell];
                    const float shx = (float)dx * M.cell - pj.x;
                    const float shy = (float)dy * M.cell - pj.y;
                    const float shz = DIM == 3 ? (float)dz * M.cell - pj.z : 0.0f;
                    const uint32_t code = vl_code<DIM>(dx, dy, dz);
                    // the cell's particles four at a time: their loads issue together (an
                    // index past the cell's end loads its last particle and is skipped)
                    for (uint32_t i0 = s; i0 < e; i0 += kVlBatch) {
                        float4 q[kVlBatch];
#pragma unroll
                        for (int u = 0; u < kVlBatch; u++) q[u] = G.P4[min(i0 + u, e - 1u)];
#pragma unroll
                        for (int u = 0; u < kVlBatch; u++) {
                            const uint32_t i = i0 + u;
                            // past the cell's end, itself, or non-existent (stays so): no candidate
                            if (i >= e || i == k || __float_as_int(q[u].w) == P.type_non_existent) continue;
                            const float ddx = q[u].x + shx, ddy = q[u].y + shy, ddz = DIM == 3 ? q[u].z + shz : 0.0f;
                            const float d2 = DIM == 3 ? ddx * ddx + ddy * ddy + ddz * ddz : ddx * ddx + ddy * ddy;
                            if (d2 < P.vl_cut2) {
                                if (nl < (uint32_t)CAP) {
                                    // shifted in: the group's entries in order once its fourth arrives
                                    buf = make_uint4(buf.y, buf.z, buf.w, i | code);
                                    if ((nl & 3u) == 3u) slab[(size_t)(nl >> 2) * P.n] = buf;
                                }
                                nl++;
                            }
                        }
                    }
                }
            }
        }
    }
    if (nl < (uint32_t)CAP && (nl & 3u)) {  // the padded last group: its m entries to the front
        const uint32_t m = nl & 3u;
        buf = m == 1u ? make_uint4(buf.w, kVlNone, kVlNone, kVlNone)
                      : (m == 2u ? make_uint4(buf.z, buf.w, kVlNone, kVlNone) : make_uint4(buf.y, buf.z, buf.w, kVlNone));
        slab[(size_t)(nl >> 2) * P.n] = buf;
    }
    G.vcount[k] = nl <= (uint32_t)CAP ? nl : kListOver;
    if (nl > (uint32_t)CAP) {  // its search needs a fresh grid each step
        atomicOr(S.vl_rebuild, 1u);
        atomicOr(S.vl_gone, 2u);
    }
}

// One candidate's contribution to the density gather: W (summation) or the
// continuity rate with its delta-SPH term (density_con, Density.h:63-114,
// the same arithmetic as k_density_mixed).
template <int DIM, int SKF, bool CONT>
__device__ __forceinline__ float density_term(const MixedF& M, int skf, float f, float dx, float dy, float dz,
                                              float d2, float4 vdi, float4 vdj, bool delta) {
    const float inv_dist = rsqrtf(d2);
    const float q = d2 * inv_dist * M.inv_h;
    if (!CONT) return SKF == 1 ? cubic_wf_sel(f, q) : kernel_wf(skf, f, q);
    const float sc = SKF == 1 ? cubic_dwdr_sel(f, q, inv_dist, M.inv_h)
                              : kernel_dwdr_scalef(skf, f, q, inv_dist, M.inv_h);
    float vcc = (vdi.x - vdj.x) * dx + (vdi.y - vdj.y) * dy;
    if (DIM == 3) vcc += (vdi.z - vdj.z) * dz;
    float term = vcc * sc;
    if (delta) {
        const float rho_factor = __fdividef(vd4_drho<DIM>(vdi, vdj), M.rho0 + vdi.w);
        term += 2.0f * M.dhc * (rho_factor * -sc);
    }
    return term;
}

// density_sum (Density.h:25-61) + EOS, or density_con (Density.h:63-114), over
// the candidate list: the entries within the cutoff are this step's
// neighbours, written to nlist for the force pass. A particle whose list
// overflowed searches the stencil cells (the grid is rebuilt every step while
// one does) and writes its neighbours too.
template <int DIM, int SKF, bool CONT>
__global__ void __launch_bounds__(kMaxGatherThreads) k_density_verlet(DevParams P, State S, Sorted G,
                                                                     StepScalars* __restrict__ scal,
                                                                     uint32_t* __restrict__ flags) {
    constexpr int CAP = Vl<DIM>::cap;
    constexpr uint32_t IDX = Vl<DIM>::index;
    // the force gather may launch now: it waits for this grid at its start (griddepcontrol.wait)
    asm volatile("griddepcontrol.launch_dependents;");
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = k < P.n;
    uint32_t cnt = 0;
    if (active) {
        const MixedF& M = P.mf;
        const uint32_t id = G.id[k];
        const float4 pj = G.P4[k];
        const int32_t tj = __float_as_int(pj.w);
        const int skf = SKF ? SKF : P.density_skf;
        const float f = M.kf[skf];
        const bool delta = CONT && P.density_treatment == 2;
        const float4 vdj = CONT ? G.VD4[k] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        Kahan acc{0.0f, 0.0f};
        uint32_t* const nslab = G.nlist + (size_t)k * 4;  // neighbour e at nslab[(e / 4) * 4n + e % 4]
        if (tj != P.type_non_existent) {
            const uint32_t vc = G.vcount[k];
            if (vc != kListOver) {
                const uint4* slab = reinterpret_cast<const uint4*>(G.vlist) + k;  // group g at slab[g * n]
                // shift of offset code (cx, cy, cz) = (cx - 2, cy - 2, cz - 2) cells, relative to this particle
                const float bx = -2.0f * M.cell - pj.x, by = -2.0f * M.cell - pj.y, bz = -2.0f * M.cell - pj.z;
                // groups of four entries (one load, the next group's issued before this
                // one's particles are loaded), then their particles, loaded together;
                // the body has no branch but the rare guard-band test, and each group's
                // sum is added with compensation
                // (list words are read once a step: streaming loads keep L1 for the neighbours' data)
                uint4 w = vc ? __ldcs(slab) : make_uint4(kVlNone, kVlNone, kVlNone, kVlNone);
                for (uint32_t e0 = 0; e0 < vc; e0 += kVlBatch) {
                    const uint4 wn = e0 + kVlBatch < vc ? __ldcs(slab + (size_t)((e0 >> 2) + 1) * P.n) : w;
                    const uint32_t en[kVlBatch] = {w.x, w.y, w.z, w.w};
                    float4 pb[kVlBatch];
#pragma unroll
                    for (int j = 0; j < kVlBatch; j++)
                        pb[j] = en[j] != kVlNone ? G.P4[en[j] & IDX] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    float part = 0.0f;
#pragma unroll
                    for (int j = 0; j < kVlBatch; j++) {
                        uint32_t cx, cy, cz;
                        vl_offset<DIM>(en[j], cx, cy, cz);
                        const float dx = pb[j].x + fmaf((float)cx, M.cell, bx);
                        const float dy = pb[j].y + fmaf((float)cy, M.cell, by);
                        const float dz = DIM == 3 ? pb[j].z + fmaf((float)cz, M.cell, bz) : 0.0f;
                        const float d2 = DIM == 3 ? dx * dx + dy * dy + dz * dz : dx * dx + dy * dy;
                        bool in = en[j] != kVlNone && __float_as_int(pb[j].w) != P.type_non_existent &&
                                  d2 < M.cut2_hi;
                        if (in && !(d2 < M.cut2_lo)) in = within_cutoff<DIM>(P, S, G, en[j] & IDX, k, d2);
                        const float4 vdi = CONT && in ? G.VD4[en[j] & IDX] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                        const float t = density_term<DIM, SKF, CONT>(M, skf, f, dx, dy, dz, d2, vdi, vdj, delta);
                        part += in ? t : 0.0f;
                        if (in) nslab[(size_t)(cnt >> 2) * 4 * P.n + (cnt & 3u)] = en[j];
                        cnt += in;
                    }
                    acc.add(M.mass * part);
                    w = wn;
                }
            } else {
                constexpr int NC = DIM == 3 ? 27 : 9;
                const Stencil<DIM> st(P, G.key[k]);
#pragma unroll 1
                for (int c = 0; c < NC; c++) {
                    uint32_t cell;
                    int sx, sy, sz;
                    if (!st.cell(c, cell, sx, sy, sz)) continue;
                    const uint32_t s = G.cell_start[cell];
                    if (s == kEmpty) continue;
                    const uint32_t e = G.cell_end[cell];
                    const float shx = (float)sx * M.cell - pj.x;
                    const float shy = (float)sy * M.cell - pj.y;
                    const float shz = DIM == 3 ? (float)sz * M.cell - pj.z : 0.0f;
                    float part = 0.0f;
                    for (uint32_t i = s; i < e; i++) {
                        if (i == k) continue;
                        const float4 pi = G.P4[i];
                        if (__float_as_int(pi.w) == P.type_non_existent) continue;
                        const float dx = pi.x + shx, dy = pi.y + shy, dz = DIM == 3 ? pi.z + shz : 0.0f;
                        const float d2 = DIM == 3 ? dx * dx + dy * dy + dz * dz : dx * dx + dy * dy;
                        if (!within_cutoff<DIM>(P, S, G, i, k, d2)) continue;
                        // this step's neighbour list too (the grid is this step's: the stencil
                        // offsets are within one cell)
                        if (cnt < (uint32_t)CAP)
                            nslab[(size_t)(cnt >> 2) * 4 * P.n + (cnt & 3u)] = i | vl_code<DIM>(sx, sy, sz);
                        cnt++;
                        const float4 vdi = CONT ? G.VD4[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                        part += density_term<DIM, SKF, CONT>(M, skf, f, dx, dy, dz, d2, vdi, vdj, delta);
                    }
                    acc.add(M.mass * part);
                }
            }
        }
        G.ncount[k] = cnt < (uint32_t)CAP ? cnt : (uint32_t)CAP;
        if (cnt > P.max_nb - 1) atomicOr(flags, RRSPH_FLAG_NEIGHBOUR_OVERFLOW);
        if (!CONT) {
            // rho - rho0 = sum - (rho0 - m W(0)): the two are within a factor of two,
            // so the float difference is exact; the Kahan and rounding residuals follow
            const float d = ((acc.s - M.rho0_minus_w0_hi) - acc.c) - M.rho0_minus_w0_lo;
            const float rho = M.rho0 + d;
            const float pr = eos_pf(M, d);
            const float2 prr = make_float2(pr, pr * __frcp_rn(rho * rho));
            if (DIM == 2)  // V4.zw = (the pressure the 2D force pass reads of a neighbour: p (form 1) or p/rho^2, rho)
                reinterpret_cast<float2*>(G.V4 + k)[1] = make_float2(P.intf_form == 1 ? prr.x : prr.y, rho);
            else
                G.V4[k].w = rho;
            G.PR[k] = prr;
            S.rho[id] = P.rho0 + f2d(d);
            S.p[id] = f2d(pr);
        } else {
            const float d = (float)(S.rho[id] - P.rho0);
            const float pr = eos_pf(M, d);
            const float rf = G.V4[k].w;  // rho_predict, the density of the forces
            const float2 prr = make_float2(pr, pr * __frcp_rn(rf * rf));
            if (DIM == 2) G.V4[k].z = P.intf_form == 1 ? prr.x : prr.y;
            G.PR[k] = prr;
            S.p[id] = pr;
            S.drho[id] = acc.value();
        }
    }
    warp_sum_add(&scal->pairs, cnt);
}

#if RRSPH_DENSITY_CELL_TILES
// The cell-tile variant of the 2D summation density pass (compile-time switch
// RRSPH_DENSITY_CELL_TILES=1; the candidate-list pass above is the default).
// Each warp (32 consecutive particles in the build's cell order, a 2x2 block
// of cells or two) stages the particles of its cells' neighbourhood, the
// bounding box of its build cells widened by two cells each way, from the
// cell table into shared memory; each lane then tests every particle of the
// build cells in its particle's window (the 3x3 to 4x4 cells k_vl_build
// searched) against the reference's cutoff, with the same float test, guard
// band and double re-test, and writes this step's neighbour list for the
// force pass as the list variant does. A warp whose box or particle count
// exceeds the stage reads the cell table and the particles from global memory
// instead. The cell table read here is the one of the last list build: with
// this variant the key pass leaves it in place (DevParams::keep_cells) and
// each rebuild clears it wholesale.
constexpr int kTileWarps = 4;         // warps per block
constexpr int kTileBoxCells = 64;     // cells of a staged box
constexpr int kTileCap = 384;         // particles of a staged box
struct TileStage {
    float4 p[kTileCap];
    uint32_t start[kTileBoxCells];    // first stage index of a box cell
    uint32_t slot0[kTileBoxCells];    // its first sorted index
    uint32_t count[kTileBoxCells];
};

template <bool STAGED>
__device__ __forceinline__ void tile_density_cells(const DevParams& P, const State& S, const Sorted& G,
                                                   const TileStage& T, uint32_t k, uint32_t cx, uint32_t cy,
                                                   uint32_t bx0, uint32_t by0, uint32_t bw, float4 pj,
                                                   Kahan& acc, uint32_t& cnt, uint4& nb, uint4* nout) {
    const MixedF& M = P.mf;
    const float f = M.kf[1];
    const float2 bo = S.boff[G.id[k]];
    int x0, x1, y0, y1;
    vl_window<2>(bo.x, cx, M.cell, P.vl_skin_edge, x0, x1);
    vl_window<2>(bo.y, cy, M.cell, P.vl_skin_edge, y0, y1);
#pragma unroll 1
    for (int dx = x0; dx <= x1; dx++) {
#pragma unroll 1
        for (int dy = y0; dy <= y1; dy++) {
            uint32_t s, c, base;
            if (STAGED) {
                const uint32_t b = (cx + dx - bx0) + (cy + dy - by0) * bw;
                c = T.count[b];
                s = T.slot0[b];
                base = T.start[b];
            } else {
                const uint32_t cell = split2_32(cx + dx) | (split2_32(cy + dy) << 1);
                if (cell >= P.max_cells) continue;
                s = G.cell_start[cell];
                if (s == kEmpty) continue;
                c = G.cell_end[cell] - s;
                base = s;
            }
            const float shx = (float)dx * M.cell - pj.x;
            const float shy = (float)dy * M.cell - pj.y;
            const uint32_t code = vl_code<2>(dx, dy, 0);
            float part = 0.0f;
            for (uint32_t t = 0; t < c; t++) {
                const uint32_t i = s + t;
                const float4 pi = STAGED ? T.p[base + t] : G.P4[base + t];
                const float ddx = pi.x + shx, ddy = pi.y + shy;
                const float d2 = ddx * ddx + ddy * ddy;
                bool in = i != k && __float_as_int(pi.w) != P.type_non_existent && d2 < M.cut2_hi;
                if (in && !(d2 < M.cut2_lo)) in = within_cutoff<2>(P, S, G, i, k, d2);
                if (in) {
                    const float inv_dist = rsqrtf(d2);
                    part += cubic_wf_sel(f, d2 * inv_dist * M.inv_h);
                    const uint32_t slot = cnt & 3u, en = i | code;
                    nb.x = slot == 0 ? en : nb.x;
                    nb.y = slot == 1 ? en : nb.y;
                    nb.z = slot == 2 ? en : nb.z;
                    nb.w = slot == 3 ? en : nb.w;
                    if (slot == 3 && cnt < (uint32_t)kVerletCap2) nout[(size_t)(cnt >> 2) * P.n] = nb;
                    cnt++;
                }
            }
            acc.add(M.mass * part);
        }
    }
}

__global__ void __launch_bounds__(kTileWarps * 32) k_density_tiles(DevParams P, State S, Sorted G,
                                                                   StepScalars* __restrict__ scal,
                                                                   uint32_t* __restrict__ flags) {
    asm volatile("griddepcontrol.launch_dependents;");
    __shared__ TileStage stage[kTileWarps];
    TileStage& T = stage[threadIdx.x >> 5];
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = k < P.n;
    // the warp's build cells and their bounding box, two cells wider each way
    uint32_t cx = 0, cy = 0;
    if (active) {
        const uint32_t key = G.key[k];
        cx = second_bits(key);
        cy = second_bits(key >> 1);
    }
    const uint32_t xmin = __reduce_min_sync(0xFFFFFFFFu, active ? cx : 0xFFFFFFFFu);
    const uint32_t xmax = __reduce_max_sync(0xFFFFFFFFu, active ? cx : 0u);
    const uint32_t ymin = __reduce_min_sync(0xFFFFFFFFu, active ? cy : 0xFFFFFFFFu);
    const uint32_t ymax = __reduce_max_sync(0xFFFFFFFFu, active ? cy : 0u);
    if (xmin == 0xFFFFFFFFu) return;  // no particle in this warp
    const uint32_t bx0 = xmin >= 2 ? xmin - 2 : 0, by0 = ymin >= 2 ? ymin - 2 : 0;
    const uint32_t bx1 = xmax + 2 <= kMaxCellCoord2 ? xmax + 2 : kMaxCellCoord2;
    const uint32_t by1 = ymax + 2 <= kMaxCellCoord2 ? ymax + 2 : kMaxCellCoord2;
    const uint32_t bw = bx1 - bx0 + 1, nbox = bw * (by1 - by0 + 1);
    bool staged = nbox <= (uint32_t)kTileBoxCells;
    if (staged) {
        // per box cell: its range in the sorted order, and an exclusive prefix
        // of the counts over the box (two rounds of 32 cells)
        uint32_t total = 0;
        for (uint32_t b0 = 0; b0 < nbox; b0 += 32) {
            const uint32_t b = b0 + lane;
            uint32_t s = 0, c = 0;
            if (b < nbox) {
                const uint32_t cell = split2_32(bx0 + b % bw) | (split2_32(by0 + b / bw) << 1);
                if (cell < P.max_cells) {
                    s = G.cell_start[cell];
                    if (s != kEmpty) c = G.cell_end[cell] - s;
                    else s = 0;
                }
            }
            uint32_t incl = c;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
                if (lane >= (uint32_t)o) incl += v;
            }
            if (b < nbox) {
                T.start[b] = total + incl - c;
                T.slot0[b] = s;
                T.count[b] = c;
            }
            total += __shfl_sync(0xFFFFFFFFu, incl, 31);
        }
        staged = total <= (uint32_t)kTileCap;
        __syncwarp();
        if (staged) {
            for (uint32_t b = lane; b < nbox; b += 32) {
                const uint32_t s = T.slot0[b], c = T.count[b], d = T.start[b];
                for (uint32_t t = 0; t < c; t++) T.p[d + t] = G.P4[s + t];
            }
        }
        __syncwarp();
    }
    uint32_t cnt = 0;
    if (active) {
        const MixedF& M = P.mf;
        const uint32_t id = G.id[k];
        const float4 pj = G.P4[k];
        Kahan acc{0.0f, 0.0f};
        uint4* const nout = reinterpret_cast<uint4*>(G.nlist) + k;  // group g at nout[g * n]
        uint4 nb = make_uint4(kVlNone, kVlNone, kVlNone, kVlNone);
        if (__float_as_int(pj.w) != P.type_non_existent) {
            if (staged) tile_density_cells<true>(P, S, G, T, k, cx, cy, bx0, by0, bw, pj, acc, cnt, nb, nout);
            else tile_density_cells<false>(P, S, G, T, k, cx, cy, bx0, by0, bw, pj, acc, cnt, nb, nout);
            if ((cnt & 3u) && cnt < (uint32_t)kVerletCap2) nout[(size_t)(cnt >> 2) * P.n] = nb;
        }
        G.ncount[k] = cnt < (uint32_t)kVerletCap2 ? cnt : (uint32_t)kVerletCap2;
        if (cnt > P.max_nb - 1) atomicOr(flags, RRSPH_FLAG_NEIGHBOUR_OVERFLOW);
        const float d = ((acc.s - M.rho0_minus_w0_hi) - acc.c) - M.rho0_minus_w0_lo;
        const float rho = M.rho0 + d;
        const float pr = eos_pf(M, d);
        const float2 prr = make_float2(pr, pr * __frcp_rn(rho * rho));
        reinterpret_cast<float2*>(G.V4 + k)[1] = make_float2(P.intf_form == 1 ? prr.x : prr.y, rho);
        G.PR[k] = prr;
        S.rho[id] = P.rho0 + f2d(d);
        S.p[id] = f2d(pr);
    }
    warp_sum_add(&scal->pairs, cnt);
}
#endif

// update_acceleration over this step's neighbours: the list the density pass
// wrote (or the stencil search for an overflowed list). In 2D a neighbour's
// pressure comes with its velocity and density (V4.z); in 3D from PR. STD: the
// common method set of ForceAcc::pair_std (2D) / pair_std3 (3D), fixed at
// compile time. At most
// 64 registers (4 blocks of 256 threads per SM): the gather hides its L1/L2
// latency with warps.
// WV != 0: the whole step follows in the same thread (whole_particle with
// variant WV, thread 0 advancing the scalars into next): it reads nothing that
// another thread's whole step writes, because this step's copies (P4, V4, VD4)
// are not the ones the key pass writes (P4n, V4n, VD4n), and the list of every
// particle is complete (the density pass wrote the neighbours of overflowed
// lists too, which needs at most Vl<DIM>::cap neighbours per particle).
template <int DIM, int SKF, bool STD, int WV>
__global__ void __launch_bounds__(kMaxGatherThreads, 4) k_forces_verlet(DevParams P, State S, Sorted G,
                                                                    StepScalars* __restrict__ scal,
                                                                    StepScalars* __restrict__ next,
                                                                    uint32_t* __restrict__ flags) {
    constexpr uint32_t IDX = Vl<DIM>::index;
    // launched while the density gather finishes: wait for it (and its writes) first
    asm volatile("griddepcontrol.wait;" ::: "memory");
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = k < P.n;
    double amag = 0, arvmu_d = 0;
    if (active) {
        const MixedF& M = P.mf;
        const uint32_t id = G.id[k];
        const float4 pj4 = G.P4[k];
        const int32_t tj = __float_as_int(pj4.w);
        ForceAcc<DIM, SKF> F{P, G, G.V4[k], G.PR[k], 0.0f, false, false, false, false, false, 0, 0,
                             0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
        F.rhoj = F.vj.w;
        F.ext = P.repulsive && tj > 0;
        F.intf = true;
        F.visc = P.art_visc;
        F.avel = P.avg_vel;
        F.form1 = P.intf_form == 1;
        F.intf_skf = SKF ? SKF : P.intf_skf;
        F.av_skf = SKF ? SKF : P.av_skf;
        Kahan ax{0, 0}, ay{0, 0}, az{0, 0};
        Kahan avx{0, 0}, avy{0, 0}, avz{0, 0};
        if (tj != P.type_non_existent) {
            const uint32_t vc = G.vcount[k];
            if (WV != 0 || vc != kListOver) {
                // this step's neighbours, four list words per load (the lanes of a
                // warp load neighbouring uint4s), their data two at a time
                const uint32_t nc = G.ncount[k];
                const uint4* nslab = reinterpret_cast<const uint4*>(G.nlist) + k;  // group g at nslab[g * n]
                const float bx = -2.0f * M.cell - pj4.x, by = -2.0f * M.cell - pj4.y, bz = -2.0f * M.cell - pj4.z;
                for (uint32_t e0 = 0; e0 < nc; e0 += 4) {
                    const uint4 w = __ldcs(nslab + (size_t)(e0 >> 2) * P.n);  // streaming, as in the density pass
                    const uint32_t eg[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
                    for (int h = 0; h < 4; h += kVlForceBatch<DIM, STD>) {
                        uint32_t en[kVlForceBatch<DIM, STD>];
                        float4 pb[kVlForceBatch<DIM, STD>], vb[kVlForceBatch<DIM, STD>];
                        float2 rb[kVlForceBatch<DIM, STD>];
#pragma unroll
                        for (int j = 0; j < kVlForceBatch<DIM, STD>; j++) en[j] = e0 + h + j < nc ? eg[h + j] : kVlNone;
#pragma unroll
                        for (int j = 0; j < kVlForceBatch<DIM, STD>; j++) {
                            if (en[j] == kVlNone) continue;
                            const uint32_t i = en[j] & IDX;
                            pb[j] = G.P4[i];
                            vb[j] = G.V4[i];
                            if (DIM == 3) rb[j] = G.PR[i];
                        }
                        // each pair's terms are added with compensation (no per-cell
                        // partial sums, whose flushes would split the warp)
#pragma unroll
                        for (int j = 0; j < kVlForceBatch<DIM, STD>; j++) {
                            if (en[j] == kVlNone) continue;
                            uint32_t cx, cy, cz;
                            vl_offset<DIM>(en[j], cx, cy, cz);
                            const float dx = pb[j].x + fmaf((float)cx, M.cell, bx);
                            const float dy = pb[j].y + fmaf((float)cy, M.cell, by);
                            const float dz = DIM == 3 ? pb[j].z + fmaf((float)cz, M.cell, bz) : 0.0f;
                            const float d2 = DIM == 3 ? dx * dx + dy * dy + dz * dz : dx * dx + dy * dy;
                            F.cax = F.cay = F.caz = F.cvx = F.cvy = F.cvz = 0.0f;
                            if (DIM == 2 && STD) {
                                F.pair_std(vb[j], dx, dy, d2, __float_as_int(pb[j].w));
                            } else if (DIM == 3 && STD) {
                                F.pair_std3(vb[j], rb[j], dx, dy, dz, d2, __float_as_int(pb[j].w));
                            } else {
                                float2 pri;
                                if (DIM == 3) {
                                    pri = rb[j];
                                } else {  // p (form 1) or p/rho^2, as the density pass wrote it
                                    const float z = vb[j].z;
                                    pri = F.form1 ? make_float2(z, z * __frcp_rn(vb[j].w * vb[j].w))
                                                  : make_float2(z, z);
                                }
                                F.pair_with(vb[j], pri, dx, dy, dz, d2, __float_as_int(pb[j].w));
                            }
                            ax.add(F.cax);
                            ay.add(F.cay);
                            if (DIM == 3) az.add(F.caz);
                            if (!STD && F.avel) {
                                avx.add(F.cvx);
                                avy.add(F.cvy);
                                if (DIM == 3) avz.add(F.cvz);
                            }
                        }
                    }
                }
            } else {
                constexpr int NC = DIM == 3 ? 27 : 9;
                const Stencil<DIM> st(P, G.key[k]);
#pragma unroll 1
                for (int c = 0; c < NC; c++) {
                    uint32_t cell;
                    int sx, sy, sz;
                    if (!st.cell(c, cell, sx, sy, sz)) continue;
                    const uint32_t s = G.cell_start[cell];
                    if (s == kEmpty) continue;
                    const uint32_t e = G.cell_end[cell];
                    const float shx = (float)sx * M.cell - pj4.x;
                    const float shy = (float)sy * M.cell - pj4.y;
                    const float shz = DIM == 3 ? (float)sz * M.cell - pj4.z : 0.0f;
                    F.cax = F.cay = F.caz = F.cvx = F.cvy = F.cvz = 0.0f;
                    for (uint32_t i = s; i < e; i++) {
                        if (i == k) continue;
                        const float4 pi4 = G.P4[i];
                        const int32_t ti = __float_as_int(pi4.w);
                        if (ti == P.type_non_existent) continue;
                        const float dx = pi4.x + shx, dy = pi4.y + shy, dz = DIM == 3 ? pi4.z + shz : 0.0f;
                        const float d2 = DIM == 3 ? dx * dx + dy * dy + dz * dz : dx * dx + dy * dy;
                        if (!within_cutoff<DIM>(P, S, G, i, k, d2)) continue;
                        F.pair(i, dx, dy, dz, d2, ti);
                    }
                    ax.add(F.cax);
                    ay.add(F.cay);
                    if (DIM == 3) az.add(F.caz);
                    if (F.avel) {
                        avx.add(F.cvx);
                        avy.add(F.cvy);
                        if (DIM == 3) avz.add(F.cvz);
                    }
                }
            }
        }
        const double axd = ax.value(), ayd = ay.value() - P.g;  // gravity along y (ExtForce.h), 2D and 3D
        const double azd = DIM == 3 ? az.value() : 0.0;
        S.ax[id] = axd;
        S.ay[id] = ayd;
        if (DIM == 3) S.az[id] = azd;
        if (F.avel) {
            S.avx[id] = avx.value();
            S.avy[id] = avy.value();
            if (DIM == 3) S.avz[id] = avz.value();
        }
        arvmu_d = F.arvmu;
        if (P.dt_reduce) amag = sqrt(axd * axd + ayd * ayd + azd * azd);
        if (WV != 0) {
            const double dt = step_dt<(WV & kVarRare) != 0>(P, scal, flags, k == 0);
            if (k == 0) advance_scalars(P, scal, next, dt);
            whole_particle<DIM, WV>(P, S, G, id, dt, scal, flags, 1, axd, ayd, azd);
        }
    }
    if (P.dt_method == 2 && P.dt_reduce) {
        warp_max_bits(&scal->amax_bits, amag);
        warp_max_bits(&scal->mumax_bits, arvmu_d);
    }
}

}  // namespace

void launch_verlet_decide(cudaGraphConditionalHandle h, const uint32_t* rebuild, cudaStream_t st) {
    k_vl_decide<<<1, 1, 0, st>>>(h, rebuild);
}
void launch_verlet_reset(uint32_t* rebuild, uint32_t* gone, unsigned long long* builds, cudaStream_t st) {
    k_vl_reset<<<1, 1, 0, st>>>(rebuild, gone, builds);
}
void launch_verlet_upload_check(uint32_t* rebuild, const uint32_t* gone, cudaStream_t st) {
    k_vl_upload_check<<<1, 1, 0, st>>>(rebuild, gone);
}
template <int DIM>
void launch_verlet_build(const DevParams& P, const State& S, const Sorted& G, cudaStream_t st) {
    constexpr int kBuildThreads = 128;
    k_vl_build<DIM><<<(P.n + kBuildThreads - 1) / kBuildThreads, kBuildThreads, 0, st>>>(P, S, G);
}
template <int DIM>
void launch_density_verlet(const DevParams& P, const State& S, const Sorted& G, StepScalars* scal, uint32_t* flags,
                           cudaStream_t st, int threads) {
    const unsigned blocks = (P.n + threads - 1) / threads;
    const bool cont = P.density_treatment != 0;
#if RRSPH_DENSITY_CELL_TILES
    if (DIM == 2 && !cont && P.all_cubic) {
        constexpr int tt = kTileWarps * 32;
        k_density_tiles<<<(P.n + tt - 1) / tt, tt, 0, st>>>(P, S, G, scal, flags);
        return;
    }
#endif
    if (P.all_cubic) {
        if (cont) k_density_verlet<DIM, 1, true><<<blocks, threads, 0, st>>>(P, S, G, scal, flags);
        else k_density_verlet<DIM, 1, false><<<blocks, threads, 0, st>>>(P, S, G, scal, flags);
    } else {
        if (cont) k_density_verlet<DIM, 0, true><<<blocks, threads, 0, st>>>(P, S, G, scal, flags);
        else k_density_verlet<DIM, 0, false><<<blocks, threads, 0, st>>>(P, S, G, scal, flags);
    }
}
// A launch that may start while the stream's previous kernel finishes
// (programmatic dependent launch); the kernel waits for it with
// griddepcontrol.wait before it reads what that kernel wrote.
template <typename... Params, typename... Args>
void launch_after(void (*kernel)(Params...), unsigned blocks, int threads, cudaStream_t st, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(blocks);
    cfg.blockDim = dim3((unsigned)threads);
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, args...);
}

template <int DIM>
void launch_forces_verlet(const DevParams& P, const State& S, const Sorted& G, StepScalars* scal,
                          StepScalars* scal_next, uint32_t* flags, cudaStream_t st, int threads, int whole) {
    const unsigned blocks = (P.n + threads - 1) / threads;
    const bool std_terms = P.all_cubic && P.intf_form != 1 && P.art_visc && !P.art_pressure && !P.avg_vel;
    const int wv = whole ? (kVarMixed | (P.density_treatment != 0 ? kVarCont : 0) |
                            (P.avg_vel || P.dt_method == 2 ? kVarRare : 0))
                         : 0;
// the force gather follows the density gather with a programmatic dependency:
// its blocks launch as the density gather's last blocks run, then wait for it
#define RRSPH_FV(SKF, STD, WV) \
    launch_after(k_forces_verlet<DIM, SKF, STD, WV>, blocks, threads, st, P, S, G, scal, scal_next, flags)
#define RRSPH_FV_WV(SKF, STD)                                                          \
    do {                                                                               \
        switch (wv) {                                                                  \
        case 0: RRSPH_FV(SKF, STD, 0); break;                                          \
        case kVarMixed: RRSPH_FV(SKF, STD, kVarMixed); break;                          \
        case kVarMixed | kVarCont: RRSPH_FV(SKF, STD, kVarMixed | kVarCont); break;    \
        case kVarMixed | kVarRare: RRSPH_FV(SKF, STD, kVarMixed | kVarRare); break;    \
        default: RRSPH_FV(SKF, STD, kVarMixed | kVarCont | kVarRare);                  \
        }                                                                              \
    } while (0)
    if (std_terms) RRSPH_FV_WV(1, true);
    else if (P.all_cubic) RRSPH_FV_WV(1, false);
    else RRSPH_FV_WV(0, false);
#undef RRSPH_FV_WV
#undef RRSPH_FV
}

namespace {

// The neighbour list the last density pass of the reuse step wrote (nlist,
// ncount: build slots with cell codes, in list order), as particle ids: row
// G.id[k] of `list` gets the ids of slot k's entries.
template <int DIM>
__global__ void k_nlist_export(DevParams P, Sorted G, uint32_t* __restrict__ counts, uint32_t* __restrict__ list,
                               uint32_t max_per, uint32_t* __restrict__ flags) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P.n) return;
    const uint32_t id = G.id[k], c = G.ncount[k];
    counts[id] = c;
    // a searched (over-full) particle stores at most the list capacity: a full
    // row may have lost entries, which this copy cannot show
    const bool clipped = c == (uint32_t)Vl<DIM>::cap && G.vcount[k] == kListOver;
    if (c > max_per || clipped) atomicOr(flags, RRSPH_FLAG_NEIGHBOUR_OVERFLOW);
    const uint32_t* const nslab = G.nlist + (size_t)k * 4;
    const uint32_t m = c < max_per ? c : max_per;
    for (uint32_t e = 0; e < m; e++)
        list[(size_t)id * max_per + e] = G.id[nslab[(size_t)(e >> 2) * 4 * P.n + (e & 3u)] & Vl<DIM>::index];
}

}  // namespace

template <int DIM>
void launch_nlist_export(const DevParams& P, const Sorted& G, uint32_t* counts, uint32_t* list, uint32_t max_per,
                         uint32_t* flags, cudaStream_t st) {
    const unsigned blocks = (P.n + 255) / 256;
    k_nlist_export<DIM><<<blocks, 256, 0, st>>>(P, G, counts, list, max_per, flags);
}

namespace {
__global__ void k_clear_cells(uint32_t* __restrict__ cell_start, uint32_t max_cells) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < max_cells) cell_start[c] = kEmpty;
}
}  // namespace

void launch_clear_cells(uint32_t* cell_start, uint32_t max_cells, cudaStream_t st) {
    k_clear_cells<<<(max_cells + 255) / 256, 256, 0, st>>>(cell_start, max_cells);
}

template void launch_nlist_export<2>(const DevParams&, const Sorted&, uint32_t*, uint32_t*, uint32_t, uint32_t*,
                                     cudaStream_t);
template void launch_nlist_export<3>(const DevParams&, const Sorted&, uint32_t*, uint32_t*, uint32_t, uint32_t*,
                                     cudaStream_t);

template void launch_verlet_build<2>(const DevParams&, const State&, const Sorted&, cudaStream_t);
template void launch_verlet_build<3>(const DevParams&, const State&, const Sorted&, cudaStream_t);
template void launch_density_verlet<2>(const DevParams&, const State&, const Sorted&, StepScalars*, uint32_t*,
                                       cudaStream_t, int);
template void launch_density_verlet<3>(const DevParams&, const State&, const Sorted&, StepScalars*, uint32_t*,
                                       cudaStream_t, int);
template void launch_forces_verlet<2>(const DevParams&, const State&, const Sorted&, StepScalars*, StepScalars*,
                                      uint32_t*, cudaStream_t, int, int);
template void launch_forces_verlet<3>(const DevParams&, const State&, const Sorted&, StepScalars*, StepScalars*,
                                      uint32_t*, cudaStream_t, int, int);

}  // namespace rrsph
