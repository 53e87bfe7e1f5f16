/*
 * CPU oracle for the exaNBody particle hot path (test infrastructure only).
 *
 * This is a restatement, in plain C++17 + OpenMP, of the reference's single-rank
 * CPU path for one velocity-Verlet molecular-dynamics step with a Lennard-Jones
 * pair functor. It is the checker against which the CUDA library is compared and
 * the timed CPU baseline; it is never linked into the product library.
 *
 * Every function in xnb_oracle.cpp names the reference file:line it follows.
 * Parity pin: the golden deck contribs/microStamp/samples/benchmark_lj_snap/
 * input_lj_Ni.msp with its check_values_lj_Ni.dat (100 sampled atoms after 100
 * steps, hex floats) is reproduced by tests/test_oracle_golden.py.
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct xo_params {
  double origin[3];      /* domain lower bound (Domain::origin, domain.h:61) */
  double extent[3];      /* domain upper bound (Domain::extent, domain.h:62) */
  int32_t dims[3];       /* domain grid dims (Domain::grid_dimension) */
  double cell_size;      /* Domain::cell_size */
  double rcut;           /* LJ cutoff (lennard_jones_force.rcut) == rcut_max */
  double rcut_inc;       /* Verlet skin (global.rcut_inc) */
  double epsilon;        /* LennardJonesParms::epsilon */
  double sigma;          /* LennardJonesParms::sigma */
  double dt;             /* global.dt */
  double mass;           /* per-type mass used by divide_force_by_type_scalar */
  int32_t divide_by_mass;/* 1: force chain ends with divide_force_by_type_scalar: mass */
  int32_t amr_enabled;   /* 1: rebuild_amr with sub_grid_density below (update-particles.msp:8-11) */
  double sub_grid_density;
} xo_params;

typedef struct xo_sys xo_sys;

xo_sys* xo_create(const xo_params* p);
void    xo_destroy(xo_sys* s);
int     xo_set_threads(int n);

/* Particles given flat; each is placed in the cell given by the periodic
 * location of its position, in input order (stable). */
int xo_load_flat(xo_sys* s, int64_t n, const double* rx, const double* ry, const double* rz,
                 const double* vx, const double* vy, const double* vz, const uint64_t* id);

/* Particles given per interior domain cell (linear index (k*Dj+j)*Di+i), in cell
 * order, as the reference lattice generator leaves them; positions may lie
 * outside their cell (init's move_particles rebins them). */
int xo_load_cells(xo_sys* s, const int64_t* cell_counts, const double* rx, const double* ry,
                  const double* rz, const double* vx, const double* vy, const double* vz,
                  const uint64_t* id);

/* Reference Ni golden-deck initial state: FCC lattice (generate_particle_lattice.h)
 * with deterministic gaussian position noise (gaussian_noise.h). Loads cells. */
int xo_load_lattice_noise_fcc(xo_sys* s, double lattice_a, double noise_sigma);
/* The same generator for structure 0 = SC, 1 = BCC, 2 = FCC. */
int xo_load_lattice_noise(xo_sys* s, int32_t structure, double lattice_a, double noise_sigma);

/* init_particles (update-particles.msp:31-36) followed by compute_all_forces_energy. */
int xo_init(xo_sys* s);
/* One numerical_scheme step (numerical-scheme.msp:21-25). Returns 1 if the
 * neighbour lists were rebuilt during this step, 0 if not, <0 on error. */
int xo_step(xo_sys* s);
int xo_compute_forces(xo_sys* s);   /* force pass alone, on an initialised state */
int xo_chunk_neighbors(xo_sys* s);  /* neighbour build alone, on an initialised state */

int64_t xo_num_particles(const xo_sys* s);
int64_t xo_rebuild_count(const xo_sys* s);
int64_t xo_num_cells(const xo_sys* s); /* interior cells */

/* Particles in storage order (interior cells in linear order, then in-cell order). */
int xo_get_particles(const xo_sys* s, double* rx, double* ry, double* rz, double* vx, double* vy,
                     double* vz, double* fx, double* fy, double* fz, uint64_t* id, int32_t* cell,
                     double* pe);
int xo_get_cell_counts(const xo_sys* s, int64_t* counts);

/* Neighbour pairs of the current lists, in list order: for each interior particle in
 * storage order, its stream entries in (cell_enc, p_b) order, as particle ids.
 * xo_pair_count gives the number of entries; xo_get_pairs fills id_a/id_b and
 * the per-particle list lengths (nbh_count, one per particle). */
int64_t xo_pair_count(const xo_sys* s);
int xo_get_pairs(const xo_sys* s, uint64_t* id_a, uint64_t* id_b, int32_t* nbh_count);
/* The same for the particles of interior cells [ci0, ci1) only (partner ids and
 * per-particle lengths), so that large systems can be compared slice by slice. */
int64_t xo_pair_count_cells(const xo_sys* s, int64_t ci0, int64_t ci1);
int xo_get_pairs_cells(const xo_sys* s, int64_t ci0, int64_t ci1, uint64_t* id_b, int32_t* nbh_count);

/* Reference-format u16 chunk stream of one interior cell (chunk_neighbors_execute.h:249-398). */
int64_t xo_cell_stream_size(const xo_sys* s, int64_t interior_cell);
int xo_get_cell_stream(const xo_sys* s, int64_t interior_cell, uint16_t* out);

/* Kinetic (0.5 m v^2) and truncated-and-shifted LJ potential energy. */
/* Particle types by id (field::type; 0 until set), ghost copies included. */
int xo_set_types(xo_sys* s, const uint64_t* ids, const uint8_t* types, int64_t n);
/* zero_particle_force + gravitational_force (contribs/pi/gravitational_force.cu:42-141)
 * over the current streams with cutoff rcut (<= the neighbour distance); masses per type. */
int xo_gravitational_force(xo_sys* s, double G, const double* type_mass, int32_t ntypes, double rcut);
/* zero_particle_force + a Morse pair potential D (exp(-2a(r-r0)) - 2 exp(-a(r-r0))),
 * shifted to 0 at rcut (<= the neighbour distance), over the current streams:
 * the user-written functor of the pair-functor API test. */
int xo_morse_force(xo_sys* s, double D, double alpha, double r0, double rcut);
/* From now on the force chain is snap_force_generic (linear SNAP, one element
 * set: chemflag, bnormflag, quadraticflag, switchinnerflag off), followed by
 * update_force_from_ghost and, when the system divides by mass, the division.
 * coeff: ntypes x ncoeffall (constant term first); forces and energies are
 * multiplied by energy_unit. with_energy: per-particle energies in pe.
 * Returns -2 when ncoeffall does not match twojmax. */
int xo_set_snap(xo_sys* s, int32_t twojmax, double rcutfac, double rfac0, double rmin0, int32_t switchflag,
                int32_t bzeroflag, int32_t ntypes, const double* radelem, const double* wj, int32_t ncoeffall,
                const double* coeff, double energy_unit, int32_t with_energy);
int xo_energy(const xo_sys* s, double* ke, double* pe);

/* Count of particles over the displacement threshold right now (particle_displ_over). */
int64_t xo_displ_over_count(const xo_sys* s);

#ifdef __cplusplus
}
#endif
