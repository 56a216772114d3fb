/*
 * abeille_gb300 — C-ABI of the GB300 multigroup transport engine.
 *
 * This is the drop-in boundary for Abeille's multigroup transport loop
 * (reference: HunterBelanger/abeille v0.4.0).  A `Transporter` subclass on the
 * reference side (`include/simulation/transporter.hpp:39-87`) hands its bank to
 * `abx_transport` and receives the fission bank back; the generation drivers
 * (`src/power_iterator.cpp:305-473`, `src/fixed_source.cpp:81-173`) map onto
 * `abx_run_power_iteration` / `abx_run_fixed_source`, which keep the bank,
 * tallies and scores resident in HBM for the whole run.
 *
 * Conventions
 *  - Every struct is plain old data; every array is caller-owned host memory,
 *    sized in elements.  No pointer handed in is retained after a call returns,
 *    except by `abx_create`, which copies everything it needs.
 *  - Every entry point returns an `int` status (ABX_OK == 0).  Nothing throws,
 *    aborts or exits across this boundary; `abx_last_error_string` returns a
 *    thread-local, human-readable description of the last failure.
 *  - Enumerations and RPN operator codes use the same numeric values as the
 *    reference, so tables built from a reference deck pass through unchanged.
 *  - A context is used by one host thread at a time and owns one CUDA stream.
 */
#ifndef ABEILLE_GB300_H
#define ABEILLE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
enum {
  ABX_OK = 0,
  ABX_ERR_INVALID = 1,       /* malformed problem or argument              */
  ABX_ERR_LOST_PARTICLE = 2, /* reference: fatal "has become lost"         */
  ABX_ERR_MAJORANT = 3,      /* reference: Et > majorant, delta_tracker.cpp:174-180 */
  ABX_ERR_OOM = 4,           /* device allocation failed                   */
  ABX_ERR_TIMEOUT = 5,       /* a bounded device wait ran out              */
  ABX_ERR_CUDA = 6,          /* any other CUDA runtime error               */
  ABX_ERR_CAPACITY = 7,      /* fission bank / secondary stack overflow    */
  ABX_ERR_NO_FISSION = 8,    /* reference: "No fission neutrons were produced." */
  ABX_ERR_UNSUPPORTED = 9,   /* feature outside the multigroup transport path */
  ABX_ERR_CANCELLED = 10,    /* request cancelled before completion        */
  ABX_ERR_BUDGET = 11        /* request does not fit the HBM admission budget */
};

/* ------------------------------------------------------------ geometry */
/* Surface kinds (reference src/{x,y,z}plane.cpp, plane.cpp, {x,y,z}cylinder.cpp, sphere.cpp).
 * Coefficients c[0..3]:
 *   XPLANE x0 | YPLANE y0 | ZPLANE z0 | PLANE A,B,C,D (Ax+By+Cz=D)
 *   XCYLINDER y0,z0,R | YCYLINDER x0,z0,R | ZCYLINDER x0,y0,R | SPHERE x0,y0,z0,R */
enum {
  ABX_SURF_XPLANE = 0,
  ABX_SURF_YPLANE = 1,
  ABX_SURF_ZPLANE = 2,
  ABX_SURF_PLANE = 3,
  ABX_SURF_XCYLINDER = 4,
  ABX_SURF_YCYLINDER = 5,
  ABX_SURF_ZCYLINDER = 6,
  ABX_SURF_SPHERE = 7
};

/* Boundary kinds, same order as the reference `enum BoundaryType`
 * (include/geometry/surfaces/surface.hpp:33). */
enum { ABX_BC_VACUUM = 0, ABX_BC_REFLECTIVE = 1, ABX_BC_NORMAL = 2 };

/* RPN operator tokens, same values as the reference `enum OP`
 * (include/geometry/cell.hpp:42-48).  Surface tokens are +-(surface index+1). */
#define ABX_OP_LPAR ((int32_t)0x7fffffff)
#define ABX_OP_RPAR ((int32_t)0x7ffffffe)
#define ABX_OP_COMP ((int32_t)0x7ffffffd)
#define ABX_OP_INTR ((int32_t)0x7ffffffc)
#define ABX_OP_UNIN ((int32_t)0x7ffffffb)

typedef struct abx_surface {
  int32_t type;     /* ABX_SURF_*                         */
  int32_t bc;       /* ABX_BC_*                           */
  uint32_t id;      /* user id (reference Surface::id)    */
  int32_t reserved;
  double c[4];
} abx_surface;

enum { ABX_FILL_MATERIAL = 0, ABX_FILL_UNIVERSE = 1 };

/* A cell: region in reverse Polish notation (reference Cell ctor takes RPN,
 * src/cell.cpp:37-67; infix->RPN is src/cell.cpp:250-299). */
typedef struct abx_cell {
  uint32_t id;
  int32_t fill_kind;  /* ABX_FILL_*                                   */
  int32_t fill;       /* material index, or universe index            */
  int32_t rpn_offset; /* first token in abx_problem.rpn               */
  int32_t rpn_len;
  int32_t reserved;
} abx_cell;

enum { ABX_UNIV_CELLS = 0, ABX_UNIV_RECT_LATTICE = 1 };

/* A universe: either a list of cells (src/cell_universe.cpp) or a rectilinear
 * lattice (src/rect_lattice.cpp).  Lattice elements are universe indices or -1,
 * ordered with index nz*(Nx*Ny) + nx*Ny + ny (src/rect_lattice.cpp:292-302). */
typedef struct abx_universe {
  uint32_t id;
  int32_t kind;        /* ABX_UNIV_*                                         */
  int32_t list_offset; /* cells: into cell_lists; lattice: into lattice_elems */
  int32_t list_len;
  int32_t shape[3];    /* lattice Nx, Ny, Nz                                 */
  int32_t outer;       /* lattice outer universe index, -1 if none           */
  double pitch[3];     /* lattice Px, Py, Pz                                 */
  double origin[3];    /* lattice centre (deck "origin")                      */
} abx_universe;

/* ------------------------------------------------------------ materials */
/* One multigroup material == one MGNuclide with atoms_bcm = 1
 * (src/material.cpp:51-63, src/mg_nuclide.cpp:579-922).  Its data live in
 * abx_problem.mg_data starting at data_offset, in this order (G = ngroups):
 *   total[G] absorption[G] fission[G] nu_prompt[G] nu_delayed[G]
 *   chi[G][G]            (a one-row deck chi is repeated for every row)
 *   scatter[G][G]        (row = incoming group, as in the deck)
 *   P1..P_L[L][G][G]     (Legendre moments, L = n_legendre, 0..5)
 *   delayed_probabilities[n_delayed] decay_constants[n_delayed]          */
typedef struct abx_material {
  uint32_t id;
  int32_t data_offset;
  int32_t n_legendre;
  int32_t n_delayed;
} abx_material;

/* ------------------------------------------------------------- tallies */
enum { ABX_EST_COLLISION = 0, ABX_EST_TRACK_LENGTH = 1 };
/* Mesh tally quantities (include/simulation/mesh_tally.hpp).  Only the ones
 * that are defined in multigroup without noise are accepted. */
enum {
  ABX_Q_FLUX = 0,
  ABX_Q_ELASTIC = 1,
  ABX_Q_ABSORPTION = 2,
  ABX_Q_FISSION = 3,
  ABX_Q_TOTAL = 4
};

typedef struct abx_mesh_tally {
  int32_t estimator;      /* ABX_EST_*                                    */
  int32_t quantity;       /* ABX_Q_*                                      */
  int32_t shape[3];       /* Nx, Ny, Nz                                   */
  int32_t ebounds_offset; /* into abx_problem.tally_ebounds               */
  int32_t n_ebounds;      /* number of energy bounds (bins + 1)           */
  int32_t reserved;
  double low[3];
  double hi[3];
} abx_mesh_tally;  /* array layout [Ne][Nx][Ny][Nz], row-major (src/mesh_tally.cpp:103-107) */

/* Shannon-entropy mesh (src/entropy.cpp, src/parser.cpp:1008-1054). */
typedef struct abx_entropy_mesh {
  int32_t enabled;
  int32_t shape[3];
  double low[3];
  double hi[3];
} abx_entropy_mesh;

/* -------------------------------------------------------------- sources */
enum { ABX_SPATIAL_POINT = 0, ABX_SPATIAL_BOX = 1 };
enum { ABX_DIR_ISOTROPIC = 0, ABX_DIR_MONO = 1 };
enum { ABX_ENERGY_MONO = 0 };

/* src/source.cpp:44-90 with src/{point,box,isotropic,mono_directional,mono_energetic}.cpp */
typedef struct abx_source {
  int32_t spatial;       /* ABX_SPATIAL_*                   */
  int32_t direction;     /* ABX_DIR_*                       */
  int32_t energy;        /* ABX_ENERGY_*                    */
  int32_t fissile_only;
  double weight;
  double low[3];         /* box low, or the point           */
  double hi[3];          /* box hi                          */
  double dir[3];         /* mono-directional direction      */
  double energy_value;   /* mono-energetic energy [MeV]     */
} abx_source;

/* ------------------------------------------------------------- settings */
enum { ABX_MODE_K_EIGENVALUE = 0, ABX_MODE_FIXED_SOURCE = 1 };
/* Transporters: DeltaTracker (src/delta_tracker.cpp), SurfaceTracker
 * (src/surface_tracker.cpp), ImplicitLeakageDeltaTracker
 * (src/implicit_leakage_delta_tracker.cpp), CarterTracker
 * (src/carter_tracker.cpp). */
enum { ABX_TRACK_DELTA = 0, ABX_TRACK_SURFACE = 1, ABX_TRACK_IMPLICIT_LEAKAGE = 2, ABX_TRACK_CARTER = 3 };
/* ABX_PREC_FP64: every operation in double, reference draw order, no FMA
 *   contraction: reproduces the reference per history.
 * ABX_PREC_MIXED: positions, directions, flight distances and cross sections
 *   in FP32; scores, tallies, k, entropy and weight normalisation in FP64;
 *   cylinder/sphere roots near grazing incidence recomputed in FP64. */
enum { ABX_PREC_FP64 = 0, ABX_PREC_MIXED = 1 };

typedef struct abx_settings {
  int32_t mode;       /* ABX_MODE_*                                        */
  int32_t tracking;   /* ABX_TRACK_*                                       */
  int32_t precision;  /* ABX_PREC_*                                        */
  int32_t ngroups;
  uint64_t seed;      /* reference default 19073486328125 (src/settings.cpp:57) */
  uint64_t stride;    /* reference default 152917        (src/settings.cpp:58) */
  double wgt_cutoff;  /* 0.25 (src/settings.cpp:62) */
  double wgt_survival;/* 1.0  (src/settings.cpp:63) */
  double nparticles;  /* tally net weight == particles per generation (src/tallies.cpp:79) */
  int32_t block_size; /* 0 = autotuned                                      */
  int32_t reserved;
  double wgt_split;   /* 2.0 (src/settings.cpp:64): Carter tracking splits a
                         particle whose |weight| reaches it                  */
  int32_t branchless; /* ABX_BRANCHLESS_* flags; non-zero with
                         ABX_MODE_K_EIGENVALUE = the reference's
                         branchless-k-eigenvalue simulation               */
  int32_t global_rng_skip; /* combing: pcg32 outputs the reference's global
                         stream (settings::rng, src/settings.cpp:59) has
                         drawn before the run -- 6 per cell and per material
                         without a colour (random plot colours,
                         src/cell.cpp:445-448, src/material.cpp:444-449) */
} abx_settings;

/* Branchless collisions (Transporter::branchless_collision,
 * src/transporter.cpp:95-267), the collisions of the reference's
 * branchless-k-eigenvalue simulation (BranchlessPowerIterator; its power
 * iteration normalises the fission bank's weights as the k-eigenvalue one
 * does).  Each collision either scatters with its weight multiplied by
 * (nu Sigma_f + Sigma_s) / Sigma_t or ends the history in one fission site of
 * that weight.  ON selects the per-nuclide form (branchless_collision_iso),
 * ON | MATERIAL the per-material one (settings branchless-material),
 * SPLITTING splits particles whose |weight| reaches wgt_split (settings
 * branchless-splitting), COMBING combs the normalised bank every generation
 * (settings branchless-combing, BranchlessPowerIterator::comb_particles,
 * src/branchless_power_iterator.cpp:592-650: std::shuffle and a comb of
 * ceil(W) equal weights drawn from the global stream, on the host between
 * generations).  Regional cancellation is not part of this path.  Delta and
 * surface tracking only; abx_create returns ABX_ERR_UNSUPPORTED for other
 * combinations. */
enum { ABX_BRANCHLESS_ON = 1, ABX_BRANCHLESS_MATERIAL = 2, ABX_BRANCHLESS_SPLITTING = 4,
       ABX_BRANCHLESS_COMBING = 8 };

/* ------------------------------------------------------------- problem */
typedef struct abx_problem {
  abx_settings settings;
  const double* energy_bounds;      /* ngroups + 1, ascending             */
  const abx_surface* surfaces;   int32_t n_surfaces;
  const abx_cell* cells;         int32_t n_cells;
  const int32_t* rpn;            int32_t n_rpn;
  const abx_universe* universes; int32_t n_universes;
  const int32_t* cell_lists;     int32_t n_cell_lists;
  const int32_t* lattice_elems;  int32_t n_lattice_elems;
  int32_t root_universe;
  const abx_material* materials; int32_t n_materials;
  const double* mg_data;         int64_t n_mg_data;
  const abx_mesh_tally* tallies; int32_t n_tallies;
  const double* tally_ebounds;   int32_t n_tally_ebounds;
  abx_entropy_mesh entropy;
  const abx_source* sources;     int32_t n_sources;
  /* Carter tracking: per-group ratio of the sampling cross section to the
   * majorant (deck "sampling-xs-ratio", src/parser.cpp:425-434); NULL = 1. */
  const double* sampling_xs_ratio;
} abx_problem;

/* ------------------------------------------------------- particle banks */
/* One history entering transport (reference Particle, include/simulation/particle.hpp:68-242).
 * rng_state is the pcg32 internal state (default stream); r_birth == r. */
typedef struct abx_particle {
  double r[3];
  double u[3];
  double E;
  double wgt;
  double wgt2;
  uint64_t history_id;
  uint64_t rng_state;
  uint64_t family_id;
} abx_particle;

/* One fission site (reference BankedParticle, include/simulation/particle.hpp:38-66,
 * transport fields only; the cancellation-only fields are not produced). */
typedef struct abx_site {
  double r[3];
  double u[3];
  double E;
  double wgt;
  double wgt2;
  uint64_t parent_history_id;
  uint64_t parent_daughter_id;
  uint64_t family_id;
} abx_site;

/* Per-generation scalar scores (reference ThreadLocalScores summed, src/tallies.cpp:100-140). */
typedef struct abx_scores {
  double k_col;
  double k_abs;
  double k_trk;
  double k_tot;
  double leakage;
  double mig_area;
  uint64_t collisions;      /* real collisions (Transporter::collision calls) */
  uint64_t flights;         /* delta: real+virtual+boundary flights; surface: flights */
  uint64_t lost;            /* particles lost at birth (warning in the reference) */
} abx_scores;

typedef struct abx_run_stats {
  int32_t generations;      /* generations actually run                     */
  int32_t active;           /* active (recorded) generations                */
  double kcol_avg, kcol_std;
  double ktrk_avg, ktrk_std;
  double leak_avg, leak_std;
  double mig_avg, mig_std;
  uint64_t collisions;      /* summed over all generations                  */
  uint64_t flights;
  uint64_t histories;
  double transport_ms;      /* device time inside transport kernels         */
  double total_ms;          /* wall time of the whole run                   */
} abx_run_stats;

typedef struct abx_context abx_ctx;

/* ------------------------------------------------------------ lifecycle */
/* Uploads a flattened problem and derives the device tables: row-normalised
 * scatter and chi CDFs (src/mg_nuclide.cpp:73-118 + libstdc++ discrete_distribution),
 * linearised Legendre angle tables (src/legendre_distribution.cpp:105-155),
 * per-group majorant (src/majorant.cpp:132-176).  Replaces the reference's
 * parser + DeltaTracker/SurfaceTracker constructors (src/parser.cpp:889-911,
 * src/delta_tracker.cpp:50-70). */
int abx_create(const abx_problem* problem, int device, abx_ctx** out);
int abx_destroy(abx_ctx* ctx);

/* The reference's multigroup YAML deck (src/parser.cpp:77-1054), read and
 * flattened natively: abx_deck_read parses `yaml_text` (the text of an
 * input_files/*.yaml deck) into an abx_problem owned by the returned handle
 * (valid until abx_deck_free), with the reference parser's conventions --
 * RPN regions, universe order, chi rows, `fissile-only` on the source entry,
 * top-level `sampling-xs-ratio`.  `precision` is ABX_PREC_*, which decks do
 * not carry.  ABX_ERR_INVALID with the reason in abx_last_error_string for a
 * deck outside the multigroup path or malformed.  abx_create_from_deck reads
 * and creates the context in one call (what the reference-side adapter of
 * the transporter uses: it holds the deck text, not a flattened problem). */
typedef struct abx_deck abx_deck;
int abx_deck_read(const char* yaml_text, int precision, abx_deck** deck, const abx_problem** problem);
int abx_deck_free(abx_deck* deck);
int abx_create_from_deck(const char* yaml_text, int precision, int device, abx_ctx** out);
const char* abx_last_error_string(void);
int abx_version(int* major, int* minor, int* patch);

/* ------------------------------------------------------ transport step */
/* Simulation::sample_sources (src/simulation.cpp:55-77): histories
 * first_history_id .. first_history_id+n-1, each on its own skip-ahead stream. */
int abx_sample_sources(abx_ctx* ctx, uint64_t first_history_id, size_t n,
                       abx_particle* out);

/* Transporter::transport (include/simulation/transporter.hpp:78-81;
 * src/delta_tracker.cpp:72-265, src/surface_tracker.cpp:40-221).
 * `kcol` is Tallies::kcol() of the previous generation (1.0 in the first).
 * `converged` is settings::converged (mesh tallies score only when set).
 * Sites come back in BankedParticle::operator< order, i.e. the order the
 * reference concatenates per-history banks.  In fixed-source mode fission
 * produces in-history secondaries and *n_sites is 0.  A batch context
 * (abx_create_batch) returns ABX_ERR_UNSUPPORTED. */
int abx_transport(abx_ctx* ctx, const abx_particle* bank, size_t n, double kcol,
                  int converged, abx_site* sites, size_t site_capacity,
                  size_t* n_sites, abx_scores* scores);

/* abx_transport without device allocation.  No counterpart in the reference.
 * For callers that cannot allocate device memory while they run: hosts whose
 * every device allocation goes through their own memory pool, loops that
 * cannot afford the device synchronisation cudaMalloc/cudaFree imply, and
 * processes at their memory budget, where a late allocation can fail.
 * `bank_dev` and `sites_dev` are device buffers the caller owns (layouts as
 * abx_particle / abx_site); *n_sites and *scores come back on the host.
 * Limits: at most 16384 histories and 65536 fission sites per call (larger
 * requests return ABX_ERR_CAPACITY, as does a fission bank that outgrows
 * `site_capacity`).  ABX_ERR_UNSUPPORTED, because their particles go on
 * per-thread stacks this entry point does not hold: fixed-source problems
 * with fissile materials (in-history secondaries), Carter tracking and
 * branchless collisions with splitting; also batch contexts.
 * All per-call scratch is one fixed 6 MB device array, reserved on every GPU
 * that loads the library and held until the process exits.  Every call uses
 * that same array, so calls that overlap on the GPU race.  The first call on
 * a device looks the array's address up.  Each call reads the step's status
 * back and synchronises the context's stream before it returns. */
int abx_transport_noalloc(abx_ctx* ctx, const abx_particle* bank_dev, size_t n,
                          double kcol, int converged, abx_site* sites_dev,
                          size_t site_capacity, size_t* n_sites,
                          abx_scores* scores);

/* MeshTally::record_generation / clear_generation (src/mesh_tally.cpp:121-152). */
int abx_tally_record_generation(abx_ctx* ctx, double multiplier);
int abx_tally_clear_generation(abx_ctx* ctx);
/* Copies tally `id` ([Ne][Nx][Ny][Nz]); any pointer may be NULL. */
int abx_tally_read(abx_ctx* ctx, int id, double* gen, double* avg, double* var,
                   int* generations);
int abx_tally_size(abx_ctx* ctx, int id, size_t* n_bins);

/* Entropy::add_point + calculate_entropy over a bank of sites (src/entropy.cpp:32-93). */
int abx_entropy(abx_ctx* ctx, const abx_site* sites, size_t n, double* entropy);

/* --------------------------------------------------- whole-run drivers */
/* PowerIterator::initialize + run (src/power_iterator.cpp:46-166, 305-473)
 * with the bank, sort, normalisation, entropy and tallies resident in HBM. */
int abx_run_power_iteration(abx_ctx* ctx, int ngenerations, int nignored,
                            abx_run_stats* stats, double* kcol_per_gen,
                            double* entropy_per_gen);
/* One record per generation of a device-resident power iteration. */
typedef struct abx_gen_record {
  double kcol;          /* Tallies::kcol() of the generation                 */
  double entropy;       /* Shannon entropy of its fission sites              */
  double step_ms;       /* device time of the whole generation step          */
  double transport_ms;  /* device time of the transport kernel               */
  uint64_t collisions, flights, histories, sites;
  uint64_t lost;        /* particles lost (mixed mode counts and kills them) */
} abx_gen_record;
/* As abx_run_power_iteration, with a per-generation record array [ngenerations]. */
int abx_run_power_iteration_ex(abx_ctx* ctx, int ngenerations, int nignored,
                               abx_run_stats* stats, abx_gen_record* per_gen);

/* The source bank the next generation would run after the last
 * abx_run_power_iteration[_ex] of the context: the reference's `bank` at
 * the end of PowerIterator::run (src/power_iterator.cpp:396-404, fission
 * sites turned into particles: normalised weights, new history ids, re-seeded
 * streams), which it can also write out as a source file
 * (src/simulation.cpp:137-175).  *n_out is its size; with out == NULL only
 * the size is returned.  *kcol_out (may be NULL) is the last generation's
 * k_col, the `kcol` a transport of this bank takes.  ABX_ERR_INVALID when no
 * power iteration ran since the banks were last written by another call
 * (transport, source sampling, fixed-source runs, the autotuner). */
int abx_read_source_bank(abx_ctx* ctx, abx_particle* out, size_t capacity,
                         size_t* n_out, double* kcol_out);

/* Start the next abx_run_power_iteration[_ex] of the context from a stored
 * source bank instead of the problem's sources: the reference's source-file
 * restart (PowerIterator::load_source_from_file,
 * src/power_iterator.cpp:60-132).  `source` holds n rows of 9 doubles, the
 * layout of the reference's "source" dataset (src/simulation.cpp:137-175):
 * x y z ux uy uz E wgt wgt2.  The rows become histories 0..n-1 (family id =
 * history id), each stream seeded at its history id, and nparticles (the
 * tallies' total weight and the bank normalisation) becomes the rounded total
 * weight, for this and later runs of the context.  The bank is kept for
 * every later run until cleared with n = 0.  The file itself is the caller's
 * to read (no HDF5 here); abx_read_source_bank gives what to write. */
int abx_set_source_bank(abx_ctx* ctx, const double* source, size_t n);

/* FixedSource::run (src/fixed_source.cpp:81-173). */
int abx_run_fixed_source(abx_ctx* ctx, int nbatches, uint64_t nparticles,
                         abx_run_stats* stats);

/* ------------------------------------------------- batches of problems */
/* Many independent fixed-source problems in one context.  Each problem keeps
 * its own geometry, materials, group structure, tallies, seed and stride, so
 * its results are the ones FixedSource::run (src/fixed_source.cpp:81-173)
 * gives for it alone: batch b of problem p transports histories
 * b*n_p .. (b+1)*n_p-1 (n_p = its settings.nparticles), each seeded by
 * skip-ahead on the problem's own stream.  The GPU transports every batch of
 * every problem in one launch, scoring each batch into its own copy of the
 * problem's tally bins, and then records the batches in order.  The
 * reference runs one problem per process; this entry point has no single
 * reference counterpart. */
typedef struct abx_problem_result {
  double leak_avg;          /* leakage per source particle, mean over batches */
  double leak_std;          /* its standard deviation (of the mean)           */
  uint64_t collisions;      /* summed over the problem's batches              */
  uint64_t flights;
  uint64_t histories;
  uint64_t lost;
  int32_t batches;
  int32_t tally_first;      /* id of the problem's first mesh tally           */
} abx_problem_result;

/* Like abx_create for `n_problems` problems.  All must be fixed-source with
 * the same tracking and precision (ABX_ERR_UNSUPPORTED otherwise).  Tally ids
 * number the problems' tallies in problem order (`tally_first` above). */
int abx_create_batch(const abx_problem* problems, int n_problems, int device, abx_ctx** out);

/* Replaces the problems of a batch context (same rules as abx_create_batch;
 * their tracking and precision must be the context's), keeping its stream and
 * reusing its device buffers where they are large enough.  On error the
 * context keeps its previous problems. */
int abx_batch_replace(abx_ctx* ctx, const abx_problem* problems, int n_problems);

/* Runs `nbatches` batches of every problem of a batch context; `results`
 * (n_problems entries, may be NULL) receives each problem's scores, `stats`
 * (may be NULL) the totals, the transport device time (`transport_ms`) and,
 * in `total_ms`, the device time of the whole batches (source sampling,
 * transport, tally and score records). */
int abx_run_fixed_source_batch(abx_ctx* ctx, int nbatches, abx_problem_result* results,
                               abx_run_stats* stats);

/* Every tally bin of a context in one copy: the bins of tally 0, then tally
 * 1, ... (the layout of abx_tally_read).  `avg` / `var` (either may be NULL)
 * hold `capacity` doubles; `n_bins` receives the total. */
int abx_tally_read_all(abx_ctx* ctx, double* avg, double* var, size_t capacity, size_t* n_bins);

/* ---------------------------------------------------------- request loop */
/* A serving loop for fixed-source problems (no reference counterpart: the
 * reference runs one deck per process).  Requests are copied at submission and
 * queued; a scheduler thread admits queued requests in arrival order into a
 * round while the estimated device footprint of everything admitted and not
 * yet finished fits the HBM budget, and `lanes` GPU threads -- each with its
 * own batch context, stream and device buffers -- run rounds side by side
 * (abx_run_fixed_source_batch with a history quantum, so the blocks of a
 * running launch retire all along and a newly admitted round's launch gets
 * their SM slots as they free up).  A request that arrives while others are
 * on the device is admitted as soon as a lane and its share of the budget are
 * free; its HBM share returns when its round ends.  Results come back through
 * abx_server_poll.  Every request's results equal those of its problem run
 * alone: batch b of a problem always transports the same histories with the
 * same per-history random streams. */
typedef struct abx_server abx_server;

typedef struct abx_server_options {
  int32_t device;
  int32_t precision;          /* ABX_PREC_*: every request must match       */
  int32_t tracking;           /* ABX_TRACK_*: every request must match      */
  int32_t nbatches;           /* FixedSource batches per request (>= 1)     */
  uint64_t hbm_budget_bytes;  /* admission budget per round; 0: 150 GB      */
  int32_t max_round_problems; /* 0: no limit                                */
  int32_t keep_tallies;       /* copy each request's tally bins back        */
  int32_t lanes;              /* rounds on the GPU at once, each in its own
                                 context and stream; 0: 3                    */
  uint32_t history_quantum;   /* histories a warp takes before its block
                                 retires and frees its SM slot; 0: 256       */
} abx_server_options;

typedef struct abx_request_result {
  uint64_t request_id;
  uint64_t tag;               /* the caller's tag from abx_server_submit    */
  int32_t status;             /* ABX_OK or this request's error             */
  int32_t round;              /* scheduling round that ran it               */
  int32_t round_problems;     /* requests in that round                     */
  int32_t n_tallies;
  uint64_t n_tally_bins;      /* bins over all its tallies                  */
  abx_problem_result result;
  double queue_ms;            /* submission -> start of its round           */
  double latency_ms;          /* submission -> result available             */
} abx_request_result;

typedef struct abx_server_stats {
  uint64_t submitted, completed, failed, rounds;
  uint64_t collisions, flights, histories;
  double busy_ms;             /* wall time spent running rounds             */
  double transport_ms;        /* device time inside transport kernels       */
  double load_ms;             /* of busy_ms: loading the round's problems   */
  double run_ms;              /*   running the batches                      */
  double readback_ms;         /*   copying tally bins back                  */
  double free_ms;             /*   freeing the context after a failed round */
} abx_server_stats;

int abx_server_create(const abx_server_options* options, abx_server** out);
/* Stops admitting, finishes the running rounds, cancels queued requests and
 * frees everything. */
int abx_server_destroy(abx_server* server);
/* Copies `problem` (fixed-source, matching the server's precision and
 * tracking) and queues it.  ABX_ERR_BUDGET when it alone exceeds the budget. */
int abx_server_submit(abx_server* server, const abx_problem* problem, uint64_t tag, uint64_t* request_id);
/* Moves up to `capacity` finished results into `out`, waiting up to
 * `timeout_ms` (0: no wait, <0: until one is available) for the first. */
int abx_server_poll(abx_server* server, abx_request_result* out, int capacity, int* n_out, int timeout_ms);
/* Tally bins (avg, var; either may be NULL) of a polled request, in its own
 * tally order; `capacity` doubles each.  Available until released. */
int abx_server_tally(abx_server* server, uint64_t request_id, double* avg, double* var, size_t capacity);
int abx_server_release(abx_server* server, uint64_t request_id);
int abx_server_get_stats(abx_server* server, abx_server_stats* stats);

/* -------------------------------------------------------- diagnostics */
/* Per-event trace of the first `n_hist` histories of the next abx_transport
 * call (test hook).  Each record: history index, event kind, rng state,
 * position, direction, group, weight.  Records go to `out` (capacity in
 * records); *n_out receives the count.  Pass n_hist = 0 to disable.  FP64
 * mode only (ABX_ERR_UNSUPPORTED on a mixed-precision context: the FP32
 * kernels carry no trace code). */
typedef struct abx_trace_rec {
  uint32_t hist;
  int32_t kind;  /* 0 flight-virtual 1 flight-real 2 leak 3 reflect 4 collision-done 5 cross
                    6 resurrect 7 lost                                               */
  int32_t group;
  int32_t cell;
  uint64_t rng_state;
  double r[3];
  double u[3];
  double wgt;
} abx_trace_rec;
int abx_set_trace(abx_ctx* ctx, uint32_t n_hist, size_t capacity);
int abx_get_trace(abx_ctx* ctx, abx_trace_rec* out, size_t capacity, size_t* n_out);

/* Device time of the most recent transport launch, in milliseconds. */
int abx_last_transport_ms(abx_ctx* ctx, double* ms);

/* Power iteration runs each generation as one launch of a captured CUDA graph
 * (the same kernels, in the same order, as the direct launches; no reference
 * counterpart).  On by default; 0 launches the kernels one by one.  Traced
 * runs always launch directly. */
int abx_set_graphs(abx_ctx* ctx, int enabled);

/* Batch runs (abx_run_fixed_source_batch; no reference counterpart): every
 * warp of the transport launch retires after taking `histories_per_warp`
 * histories and the launch gets as many blocks as that needs, so blocks
 * finish throughout the run and their SM slots go to whatever else is
 * queued on the GPU -- the launches of other contexts' streams in the
 * request loop.  0 (the default): persistent warps, one wave of blocks.
 * Not applied to problems whose histories carry secondaries.  Results do
 * not depend on it. */
int abx_set_history_quantum(abx_ctx* ctx, uint32_t histories_per_warp);

/* Transport kernel (no reference counterpart; results do not depend on it).
 * HISTORY: one lane per history, the lanes of a warp running their event
 * machines side by side.  POOL: each warp keeps 128 histories in device
 * memory and runs one event kind at a time on up to 32 of them (event-sorted
 * execution inside one persistent launch); delta and surface tracking with
 * branching collisions only -- Carter tracking, branchless collisions and
 * problems whose histories carry secondaries (fixed source with fission)
 * return ABX_ERR_UNSUPPORTED.  AUTO: the engine's choice.  Setting a kernel
 * resets the launch shape to that kernel's full occupancy. */
enum {
  ABX_TRANSPORT_KERNEL_AUTO = 0,
  ABX_TRANSPORT_KERNEL_HISTORY = 1,
  ABX_TRANSPORT_KERNEL_POOL = 2
};
int abx_set_transport_kernel(abx_ctx* ctx, int kind);
/* The kernel the next transport launch uses (HISTORY or POOL). */
int abx_get_transport_kernel(abx_ctx* ctx, int* kind);

/* Launch-shape autotuner (no reference counterpart): transports the same
 * `n_probe` first-generation source histories three times per candidate
 * shape (128 or 256 threads per block, 1 .. the occupancy limit of blocks per
 * SM), scoring tallies into scratch bins, and keeps the fastest for the
 * context.  Results do not depend on the shape.  Outputs may be NULL. */
int abx_autotune(abx_ctx* ctx, size_t n_probe, int* block, int* grid, double* best_ms);

/* Timing hygiene for benchmarks (no reference counterpart): before each
 * generation of abx_run_power_iteration[_ex], outside the generation's timed
 * events, write `bytes` of a private device buffer so that the L2 cache holds
 * none of the previous generation's data.  0 (the default) turns it off. */
int abx_set_l2_flush(abx_ctx* ctx, size_t bytes);

#ifdef __cplusplus
}
#endif

#endif /* ABEILLE_GB300_H */
