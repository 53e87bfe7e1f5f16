// Host-side launchers of the xnb kernels (internal; the public C ABI is include/xnb_gpu.h).
#pragma once
#include <string>

#include "xnb_internal.cuh"

namespace xnb {

enum Precision : int { kFp64Exact = 0, kFp64 = 1, kMixed = 2 };

// Every launcher returns the number of kernels it enqueued.

// Work extent of a batch: high-water marks of the particle and cell pools.
struct Extent {
  uint32_t n_part;   // particles [0, n_part) are scanned; free slots have pcell == ~0u
  uint32_t n_cells;  // cells [0, n_cells); free cells have cell_sys == ~0u
  int nsys;
  int sm_count;
  int force_block;   // threads per block of the force traversal (multiple of 32, <= 256)
  int force_lanes;   // threads per particle of the FP64 / mixed full-list traversal (1, 2 or 4)
  int far_coords;    // some resident system lies far from the coordinate origin (SysDesc::far_coords)
  int unpacked;      // some resident system reads the residual mirror, not packed residuals (SysDesc::packed_lo)
  int force_form;    // kForceThread or kForceStaged (mixed full-list traversal)
  uint32_t n_seg;    // cell segments of the staged traversal (DevArrays::seg)
};

// Mixed-precision force traversal forms: one thread per particle over global
// memory, or cell segments staged in shared memory (xnb_force_staged.cu).
constexpr int kForceThread = 0;
constexpr int kForceStaged = 1;
constexpr int kStagedSegCells = 8;  // x-adjacent cells of one row per staged segment

// Fused first half of velocity Verlet plus the displacement trigger:
// push_f_v_r(dt_scale 1) ; push_f_v(dt_scale 0.5) ; particle_displ_over.
int launch_first_half(const Extent& ex, const SysDesc* sys, SysState* st, const DevArrays& a,
                       bool do_push_r, bool do_push_v, bool do_trigger, double dt_scale_r,
                       double dt_scale_v, bool exact, int sys_only, cudaStream_t stream);

// zero_particle_force + lennard_jones_force (+ divide_force_by_type_scalar when the
// system asks for it), optionally fused with the second-half kick push_f_v(0.5).
// newton: FP64 / mixed paths walk the lower half of each list and deliver
// reactions with FP64 reductions (three kernels: zero, traverse, finish).
int launch_force(const Extent& ex, const SysDesc* sys, SysState* st, const DevArrays& a, int precision,
                 bool with_pe, bool second_half, int sys_only, cudaStream_t stream, bool newton = false);

// Compact list entries of the flagged systems after a build, and the staged
// mixed force traversal (+ kick) over the cell segments (xnb_force_staged.cu).
// all = true: every resident system's current lists (when the staged form is switched on)
int launch_compact_lists(const Extent& ex, const SysDesc* sys, SysState* st, const DevArrays& a, cudaStream_t stream,
                         bool all = false);
int launch_force_staged(const Extent& ex, const SysDesc* sys, SysState* st, const DevArrays& a, bool with_pe,
                        bool second_half, int sys_only, cudaStream_t stream);
size_t staged_smem_bytes();

// Marks systems for rebuild: all of them (init), or those with moved > 0.
int launch_mark_rebuild(const Extent& ex, SysState* st, int mode, int sys_only, unsigned int* any,
                        cudaStream_t stream);
int launch_clear_moved(const Extent& ex, SysState* st, cudaStream_t stream);

// Control block of the persistent step loop (device memory, zeroed before each launch).
struct StepCtl {
  unsigned int arrive;      // grid barrier: blocks arrived at the current barrier
  unsigned int generation;  // grid barrier: barriers completed
  unsigned int fired[2];    // per step parity: an armed system's displacement trigger fired
  unsigned int steps_done;  // whole steps completed by the launch
  unsigned int stopped;     // 1: stopped after the first half of step steps_done (the trigger fired)
  unsigned int error;       // 1: a barrier wait ran out
  unsigned int pad;
};
// Up to max_steps whole MD steps (first half + trigger, grid barrier, forces with
// the second-half kick, grid barrier) in one cooperative launch, one thread per
// particle, full lists; it stops after the first half of a step whose trigger
// fired. check: the first barrier waits for one block more than the launch has,
// so every wait runs out after wait_ns and the launch returns before changing
// any state (a test of the timeout path). Returns the number of launches.
int launch_steps_persistent(const Extent& ex, const SysDesc* sys, SysState* st, const DevArrays& a, int precision,
                            bool with_pe, StepCtl* ctl, int max_steps, bool check, cudaStream_t stream);

// move_particles + migrate + rebuild_amr + backup_r for systems with rebuild != 0.
// exact_backup = false keeps the backup position unencoded (FP64 and mixed paths).
int launch_rebin(const Extent& ex, const SysDesc* sys, SysState* st, const DevArrays& a, cudaStream_t stream,
                 bool exact_backup = true);
// backup_r alone.
int launch_backup(const Extent& ex, const SysDesc* sys, SysState* st, const DevArrays& a, cudaStream_t stream);
// chunk_neighbors for systems with rebuild != 0: one pass writing each list
// into its particle's slot (statistics reset, the warp-per-cell build, and the
// block-per-cell build of the cells too large for it: three kernels). lbuf: the
// largest slot rounded up to 32 entries, 0 above 1024 or when no system has a
// slot yet; it sizes the shared-memory list buffers.
// form: kBuildRows (lane per particle, rows of three cells bulk-copied into
// shared memory, xnb_build_rows.cu) or kBuildWarp (lane per candidate, the
// 27-cell block staged per warp); cells neither handles go to the
// block-per-cell build.
// prune: cells with a sub-grid go to the sub-cell pruned build (xnb_build_sub.cu)
// when their system's sub-cell keys still describe its positions (keys_fresh:
// set by the rebin, cleared when positions are pushed).
constexpr int kBuildRows = 0;
constexpr int kBuildWarp = 1;
constexpr int kBuildHalf = 2;
int launch_neighbors(const Extent& ex, const SysDesc* sys, SysState* st, const DevArrays& a, int stage_cap,
                     int lbuf, cudaStream_t stream, int form = kBuildRows, bool prune = false);
// the lane-per-particle build alone (cells it cannot take are appended to a.nbr_wide)
int launch_neighbors_rows(const Extent& ex, const SysDesc* sys, SysState* st, const DevArrays& a, cudaStream_t stream,
                          bool prune);
// the half-shell build (xnb_build_half.cu): pair masks of the systems whose
// cells all hold at most 64 particles, then the lists from the masks
int launch_neighbors_half_test(const Extent& ex, const SysDesc* sys, SysState* st, const DevArrays& a,
                               cudaStream_t stream);
int launch_neighbors_half_emit(const Extent& ex, const SysDesc* sys, SysState* st, const DevArrays& a,
                               cudaStream_t stream);
// the sub-cell pruned build of the cells listed in a.nbr_sub (cells with a
// neighbour of sub-grid side above 3 are passed on to a.nbr_wide)
int launch_neighbors_sub(const Extent& ex, const SysDesc* sys, SysState* st, const DevArrays& a, int stage_cap,
                         cudaStream_t stream);

// Reference-format chunk-neighbour streams of system sid (xnb_stream.cu):
// per-cell lengths (u16 units), the streams at cell_off, and the checker
// (counts[6]: format, order, self, range, far, missing).
int launch_stream_lengths(uint32_t sid, uint32_t ncells, const SysDesc* sys, const DevArrays& a, int T,
                          uint32_t* cell_len, int sm_count, cudaStream_t stream);
int launch_stream_write(uint32_t sid, uint32_t ncells, const SysDesc* sys, const DevArrays& a, int T,
                        const unsigned long long* cell_off, uint16_t* out, unsigned int* errors, int sm_count,
                        cudaStream_t stream);
int launch_stream_verify(uint32_t sid, uint32_t ncells, const SysDesc* sys, const DevArrays& a, int T,
                         const uint16_t* stream_data, uint64_t stream_len, const unsigned long long* cell_off,
                         unsigned long long* counts, int sm_count, cudaStream_t stream);

// On-device observables (xnb_observe.cu): simulation_stats of system sid into a
// scratch area of stats_scratch_bytes() (copy_stats reads it back: kinetic
// sum, potential, min/max |v|, min/max |f| and the count), and id sampling.
size_t stats_scratch_bytes();
int launch_stats(uint32_t sid, uint32_t npart, const SysDesc* sys, const DevArrays& a, void* scratch, int sm_count,
                 cudaStream_t stream);
int copy_stats(void* scratch, double* out6, unsigned long long* count_out, cudaStream_t stream);
int launch_sample(uint32_t sid, uint32_t npart, const SysDesc* sys, const DevArrays& a, const uint64_t* ids,
                  uint32_t n, double* out, int32_t* found, int sm_count, cudaStream_t stream);

// gravitational_force over the per-particle lists (xnb_functors.cu). Masses per
// particle type (at most kMaxTypes); pre_hi_f = rcut^2 + the FP32 prefilter's
// proven margin. flags bit 0: a particle type without a mass.
constexpr int kMaxTypes = 16;
struct GravParams {
  double G;
  double rcut2;
  float pre_hi_f;
  int ntypes;
  double mass[kMaxTypes];
};
int launch_gravity(const Extent& ex, const SysDesc* sys, const SysState* st, const DevArrays& a, int precision,
                   bool with_pe, bool accumulate, int sys_only, const GravParams& gp, unsigned int* flags,
                   cudaStream_t stream);
// field::type by id for system sid (ids sorted ascending); matched += particles found
int launch_set_types(uint32_t sid, uint32_t npart, const SysDesc* sys, const DevArrays& a, const uint64_t* ids,
                     const uint8_t* types, uint32_t n, unsigned long long* matched, int sm_count, cudaStream_t stream);

// Device placement of a system uploaded in input order into the rebin scratch
// (xnb_place.cu). flags: bit 0 a position outside any representable cell, bit 1
// a cell above kPlaceMaxCell particles (the host then places the system).
constexpr uint32_t kPlaceMaxCell = 4096;
struct PlaceArgs {
  double origin[3];
  double cell_size;
  int dims[3];
  uint32_t poff, coff, n, ncells, sys_slot;
};
int launch_place(const PlaceArgs& P, const DevArrays& a, unsigned int* flags, int sm_count, cudaStream_t stream);

// Exclusive scan of u32 counts into u64 offsets (n elements; out has n+1 entries).
// With gate != nullptr the kernels return at once while *gate == 0.
int launch_scan_u32_to_u64(const uint32_t* in, unsigned long long* out, uint32_t n,
                           unsigned long long* block_scratch, cudaStream_t stream,
                           const unsigned int* gate = nullptr);
size_t scan_scratch_elems(uint32_t n);


// Allocation-free neighbour build of one system (xnb_static_scratch.cu): scratch
// in a file-scope device array; returns 0, -1 (size above the array's limit,
// *err says which) or -2 (CUDA error). cap is clamped to 2^32 - 1 entries.
int launch_neighbors_static(const SysDesc& S, uint64_t ncells, uint64_t n, const double* rx, const double* ry,
                            const double* rz, const uint32_t* cell_start, const uint32_t* cell_n, uint32_t* nbr,
                            uint64_t cap, uint32_t* nbr_start, uint32_t* nbr_cnt, unsigned long long* total_out,
                            cudaStream_t stream, std::string* err);

}  // namespace xnb
