// kernels.cuh — device buffers of a solver and the launchers of its kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

namespace rrsph {

// Particle state in id order (the reference's arrays), double precision.
struct State {
    double *rx, *ry, *rz;      // positions
    double *vx, *vy, *vz;      // velocities
    double *ax, *ay, *az;      // accelerations of the last force evaluation
    double *avx, *avy, *avz;   // XSPH average velocity (average_velocity only)
    double *vpx, *vpy, *vpz;   // v_predict
    double *rho, *p, *drho, *rho_pred;
    double *mu;                // max |mu_ij| per particle (rrsph_forces only)
    int32_t* itype;
    uint32_t* key_of;          // cell key used by the last grid build, per id
    int32_t* wave_tank;        // piston of each particle in wave_law, -1 for none (null: the params' wave maker)
    const PistonLaw* wave_law; // wave-maker table
    // FP32-mixed step only (null otherwise), written by the key pass, id order:
    float2* coff2;             // 2D: offset of r from its cell's lower edge
    float4* coff4;             // 3D: the same (x, y, z)
    float2* vpf2;              // 2D: v_predict in float
    float4* vpf4;              // 3D: the same (x, y, z)
    // mixed step with neighbour reuse (null otherwise), id order:
    uint32_t* cxy;             // cell coordinates of the current position, x | y << 16 (3D: x | y << 10 | z << 20)
    uint32_t* bcxy;            // cell coordinates at the last list build
    uint32_t* slot;            // cell-order index at the last list build
    float2* boff;              // 2D: offset from that cell's edges at the last list build
    float4* boff4;             // 3D: the same (x, y, z)
    uint32_t* vl_rebuild;      // non-zero: the next step rebuilds the grid and the lists
    uint32_t* vl_gone;         // the last build: bit 0 left out non-existent particles, bit 1 overflowed a list
    uint32_t* itype_changed;   // non-zero once a step changed a particle's type since the last upload
};

// Per-step cell-ordered copies and the grid.
struct Sorted {
    uint32_t *keys_in, *ids_in;       // key pass output (id order)
    uint32_t *keys_a, *ids_a, *keys_b, *ids_b;
    uint32_t* sort_scratch;
    uint32_t *key, *id;               // sorted result (points into a or b)
    uint32_t *cell_start, *cell_end;  // [max_cells]
    // FP64 gathers
    double *rx, *ry, *rz;
    double *vx, *vy, *vz;             // velocity the forces use (v_predict in the loop)
    double *vdx, *vdy, *vdz;          // velocity of density_con (v)
    double *rho;                      // density the forces use
    double *rhod;                     // density of density_con
    double* p;
    double* pr2;                      // p / (rho * rho) with the density the forces use (the density pass writes it)
    int32_t* itype;
    // FP32-mixed gathers
    float4* P4;    // cell-relative position (x, y, z) + itype bits
    float4* V4;    // velocity the forces use + density the forces use
    float4* VD4;   // v + (rho - rho0) for density_con
    float2* PR;    // pressure p and p / rho^2 (rho = the density the forces use)
    // mixed step with neighbour reuse: the P4 / V4 (/ VD4 with continuity
    // density) of the next step, which the key pass writes at each particle's
    // build slot (the two buffers alternate)
    float4* P4n;
    float4* V4n;
    float4* VD4n;
    // Neighbour masks written by the density pass for the force pass (the FP64
    // step, 2D and 3D; the 2D mixed step without reuse), SoA [NC + 1][n] with
    // NC = 3^dim stencil cells, of 32-bit words (64-bit in the 3D FP64 step):
    // word c < NC = bit b set if particle cell_start + b of stencil cell c is a
    // neighbour; word NC = stencil cells with more particles than a word has
    // bits (searched again by the force pass). Null where unused.
    uint32_t* nbmask;
    // mixed step with neighbour reuse: up to kVerletCap2 (2D) / kVerletCap3 (3D)
    // candidates per particle, sorted index | cell code << 27 (3D: << 25) with
    // code = (dx + 2) * 5 + (dy + 2) (3D: ((dx + 2) * 5 + (dy + 2)) * 5 + (dz + 2))
    // for the candidate's cell offset, stored in slabs of four: entries 4g..4g+3
    // of particle k are the uint4 at (uint4*)list + g * n + k (the lanes of a
    // warp read neighbouring uint4s), the last group padded with kVlNone;
    // vcount[k] = candidates (kListOver: too many, searched instead). This
    // step's neighbours (the candidates within the cutoff, in list order) in the
    // same slab layout: nlist, ncount[k] of them; words past ncount are stale.
    uint32_t* vlist;
    uint32_t* vcount;
    uint32_t* nlist;
    uint32_t* ncount;
};

// Sources the reorder gathers for the force velocity / density.
struct GatherSrc {
    const double *vx, *vy, *vz;
    const double* rho;
    const double* p;  // pressure to copy (rrsph_forces on the given state); null in the loop
    int loop;         // 1: the loop's mixed step (float v_predict from the key pass; no double copies)
};

template <int DIM>
void launch_keys(const DevParams& P, const State& S, Sorted& G, StepScalars* scal, int predict, uint32_t* flags,
                 cudaStream_t st);
template <int DIM>
void launch_reorder(const DevParams& P, const State& S, const Sorted& G, GatherSrc fsrc, int mixed, cudaStream_t st);
// The pair gathers take their block size (threads, <= kMaxGatherThreads, a
// multiple of 32) from the caller; the autotuner picks it.
template <int DIM>
void launch_density_fp64(const DevParams& P, const State& S, const Sorted& G, StepScalars* scal, uint32_t* flags,
                         cudaStream_t st, int threads);
// use_masks: the pairs are those the density pass on this grid recorded in
// G.nbmask (the same pairs in the same order as the search).
template <int DIM>
void launch_forces_fp64(const DevParams& P, const State& S, const Sorted& G, uint32_t terms, StepScalars* scal,
                        uint32_t* flags, int write_mu, cudaStream_t st, int threads, int use_masks = 0);
template <int DIM>
void launch_density_mixed(const DevParams& P, const State& S, const Sorted& G, StepScalars* scal, uint32_t* flags,
                          cudaStream_t st, int threads);
template <int DIM>
void launch_forces_mixed(const DevParams& P, const State& S, const Sorted& G, uint32_t terms, StepScalars* scal,
                         uint32_t* flags, int write_mu, int use_masks, cudaStream_t st, int threads);
// whole_step; with next_keys also the next step's predict_half_step and key pass.
template <int DIM>
void launch_whole_step(const DevParams& P, const State& S, const Sorted& G, StepScalars* scal_cur,
                       StepScalars* scal_next, uint32_t* flags, int next_keys, cudaStream_t st);

// Neighbour reuse (the FP32-mixed step): the candidate lists
// are built with the cutoff widened by a skin and reused while no particle has
// moved more than half the skin since the build (kernels_reuse.cu).
void launch_verlet_decide(cudaGraphConditionalHandle h, const uint32_t* rebuild, cudaStream_t st);
void launch_verlet_reset(uint32_t* rebuild, uint32_t* gone, unsigned long long* builds, cudaStream_t st);
// After an upload: the lists stay valid unless the last build left out a
// non-existent particle (which may exist now); moves are checked by the key pass.
void launch_verlet_upload_check(uint32_t* rebuild, const uint32_t* gone, cudaStream_t st);
template <int DIM>
void launch_verlet_build(const DevParams& P, const State& S, const Sorted& G, cudaStream_t st);
// Marks every cell-table entry empty (a kernel, so that it can sit in the
// rebuild body of a step graph's conditional node).
void launch_clear_cells(uint32_t* cell_start, uint32_t max_cells, cudaStream_t st);
// The last reuse step's neighbour list (nlist / ncount) as particle ids:
// counts[id], list[id * max_per + e]; more than max_per raises the overflow flag.
template <int DIM>
void launch_nlist_export(const DevParams& P, const Sorted& G, uint32_t* counts, uint32_t* list, uint32_t max_per,
                         uint32_t* flags, cudaStream_t st);
template <int DIM>
void launch_density_verlet(const DevParams& P, const State& S, const Sorted& G, StepScalars* scal, uint32_t* flags,
                           cudaStream_t st, int threads);
// whole != 0: the whole step of each particle (launch_whole_step with next keys)
// runs in the force gather's thread; needs dt without the step's reduction and
// at most verlet_cap(dim) + 1 neighbours per particle (max_nb).
template <int DIM>
void launch_forces_verlet(const DevParams& P, const State& S, const Sorted& G, StepScalars* scal,
                          StepScalars* scal_next, uint32_t* flags, cudaStream_t st, int threads, int whole);

void launch_cells_start(const DevParams& P, const Sorted& G, uint32_t* out, cudaStream_t st);
template <int DIM>
void launch_neighbour_list(const DevParams& P, const Sorted& G, uint32_t* counts, uint32_t* list, uint32_t max_per,
                           uint32_t* flags, cudaStream_t st);
template <int DIM>
void launch_unpack(const DevParams& P, State S, const double* r, const double* v, uint32_t stride, cudaStream_t st);
template <int DIM>
void launch_pack(const DevParams& P, State S, double* r, double* v, uint32_t stride, cudaStream_t st);
// The time of the next step (and flags cleared, when non-null); after steps,
// the time and flags into a mapped host mailbox (device address `out`).
struct HostReport {
    double time;
    uint32_t flags;
    unsigned long long pairs_last;   // directed pairs of the last completed step (0: none since upload)
    unsigned long long pairs_total;  // summed over the steps since upload
};
void launch_set_time(StepScalars* scal, double time, uint32_t* flags, cudaStream_t st);
// rrsph_diagnostics: blocks partial sums of kDiagQuantities doubles into part
// (blocks * kDiagQuantities), then their fixed-order sum into out.
constexpr int kDiagQuantities = 10;
template <int DIM>
void launch_diagnostics(const DevParams& P, const State& S, double* part, int blocks, double* out, cudaStream_t st);
// scal: the next step's scalars; last: the completed step's (null: none since upload).
void launch_report(const StepScalars* scal, const StepScalars* last, const uint32_t* flags, HostReport* out,
                   cudaStream_t st);
// Upload / download through device-addressable host arrays (pinned memory):
// one kernel reading (writing) the caller's arrays over the host link. The
// upload also runs the first step's predict + key pass (launch_keys).
template <int DIM>
void launch_upload_direct(const DevParams& P, const State& S, const Sorted& G, const double* r, const double* v,
                          const double* rho, const double* p, const int32_t* itype, uint32_t stride,
                          StepScalars* scal, double dt, uint32_t* flags, cudaStream_t st);
// itype_if (optional): itype is written only if that device word is non-zero.
template <int DIM>
void launch_download_direct(const DevParams& P, const State& S, double* r, double* v, double* rho, double* p,
                            int32_t* itype, uint32_t stride, cudaStream_t st, const uint32_t* itype_if = nullptr);

// Compile-time variant: the cell-tile density pass of the 2D mixed step with
// neighbour reuse (summation density, cubic kernel) instead of the
// candidate-list pass (kernels_reuse.cu).
#ifndef RRSPH_DENSITY_CELL_TILES
#define RRSPH_DENSITY_CELL_TILES 0
#endif
constexpr int kVerletCap2 = 64;         // candidate-list entries per particle, 2D
constexpr int kVerletCap3 = 256;        // and 3D
inline int verlet_cap(int dim) { return dim == 3 ? kVerletCap3 : kVerletCap2; }
// particles a list entry can index (the cell code takes the top bits)
inline uint64_t verlet_max_particles(int dim) { return dim == 3 ? (1ull << 25) : (1ull << 27); }
constexpr uint32_t kListOver = 0xFFFFFFFFu;
constexpr uint32_t kVlNone = 0xFFFFFFFFu;  // padding of a list row (never an entry)
constexpr int kGatherThreads = 128;     // default block size of the pair gathers
constexpr int kMaxGatherThreads = 256;

}  // namespace rrsph
