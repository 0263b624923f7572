/* gomc_gb300.h -- C ABI of the GB300 Monte Carlo energy path.
 *
 * One gb_box is one orthogonal periodic simulation box whose coordinates,
 * cell grid, Ewald k-vectors and structure factors, and running energies stay
 * resident in HBM on one GPU.  Every call returns 0 on success or a gb_status
 * code; gb_last_error() gives the message.  No call exits the process.
 * Calls on one box are not re-entrant; separate boxes may be used from
 * separate threads.  Positions are Angstrom, energies Kelvin, charges e.
 *
 * Each entry point names the reference interface it replaces (GOMC 2.80,
 * file:line within the GOMC source tree).
 */
#ifndef GOMC_GB300_H
#define GOMC_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gb_box gb_box;

enum gb_status {
  GB_OK = 0,
  GB_ERR_ARG = 1,         /* invalid argument */
  GB_ERR_CUDA = 2,        /* CUDA runtime error */
  GB_ERR_NOMEM = 3,       /* device allocation failed */
  GB_ERR_CAPACITY = 4,    /* a cell ran out of slots */
  GB_ERR_TIMEOUT = 5,     /* a bounded device-side wait gave up */
  GB_ERR_STATE = 6,       /* call not valid in the current state */
  GB_ERR_UNSUPPORTED = 7  /* input outside what this build handles */
};

enum gb_precision { GB_FP64 = 0, GB_MIXED = 1 };

/* The molecular system of one box (what Molecules / MoleculeKind /
 * Coordinates / FFParticle hold in the reference: src/Molecules.h,
 * src/MoleculeKind.h, src/Coordinates.cpp:12-22, src/FFParticle.cpp:56-84). */
typedef struct gb_system_desc {
  int32_t n_atoms, n_mol, n_kinds;
  const double *pos;          /* [n_atoms * 3] as read from the PDB */
  const int32_t *atom_kind;   /* [n_atoms], 0 .. n_kinds-1 */
  const double *atom_charge;  /* [n_atoms] */
  const int32_t *mol_start;   /* [n_mol + 1] */
  const double *kind_epsilon; /* [n_kinds] K */
  const double *kind_sigma;   /* [n_kinds] A */
  const double *kind_n;       /* [n_kinds] Mie repulsion exponent */
  double box[3];              /* orthogonal edge lengths, A */
} gb_system_desc;

/* The in.conf keys of the energy path (src/ConfigSetup.cpp:222-1409). */
typedef struct gb_config {
  double temperature;   /* Temperature */
  double rcut;          /* Rcut */
  double rcut_low;      /* RcutLow */
  double rcut_coulomb;  /* RcutCoulomb (defaults to Rcut when <= 0) */
  double tolerance;     /* Tolerance */
  int32_t ewald;        /* Ewald */
  int32_t electrostatic;/* ElectroStatic */
  int32_t precision;    /* GB300Precision: GB_FP64 or GB_MIXED */
  int32_t device;       /* CUDA device ordinal */
  /* soft-core settings of pair terms at lambda < 1 (FreeEnergyCalc /
   * NeMTMC blocks: ScaleAlpha, ScaleSigma, ScalePower, ScaleCoulomb; all 0
   * when neither is enabled, src/Forcefield.cpp:59-75) */
  double sc_alpha, sc_sigma;
  int32_t sc_power, sc_coul;
} gb_config;

const char *gb_version(void);
const char *gb_last_error(const gb_box *box); /* NULL box: last create error */

/* System::Init (src/System.cpp:67-100): wrap coordinates into the box
 * (Coordinates::WrapCoordinate, src/Coordinates.cpp:24-73), molecule centres
 * (COM::CalcCOM, src/COM.h:47-68), CellList::GridAll
 * (src/CellList.cpp:220-237), Ewald::Init (src/Ewald.cpp:100-139) and the
 * initial CalculateEnergy::SystemTotal (src/CalculateEnergy.cpp:83-138). */
int gb_box_create(const gb_system_desc *sys, const gb_config *cfg,
                  gb_box **out);
void gb_box_destroy(gb_box *box);

/* ---- CalculateEnergy (src/CalculateEnergy.h:48-293) ---- */
/* SystemTotal: out9 = inter, real, recip, self, correction, tailCorrection,
 * intraBond, intraNonbond, total; also resets the running energies. */
int gb_system_total(gb_box *box, double *out9);
/* BoxInter (src/CalculateEnergy.cpp:157-266): LJ and real-space Coulomb */
int gb_box_inter(gb_box *box, double *inter, double *real);
/* MoleculeInter (src/CalculateEnergy.cpp:581-686): energy change of moving
 * molecule `mol` from its current position to new_pos[n_atoms_of_mol * 3]. */
int gb_molecule_inter(gb_box *box, int32_t mol, const double *new_pos,
                      double *lj, double *real, int32_t *overlap);
/* VirialCalc (src/CalculateEnergy.cpp:411-579) with Ewald::VirialReciprocal
 * (src/Ewald.cpp:1168-1305), long-range correction off: out16 = inter,
 * real, recip, total virial (K), then the xx, yy, zz diagonals of
 * interTens, realTens, recipTens, totalTens (the reference computes no
 * off-diagonal components).  Pressure (bar) = 138.0649 (N_mol T + total/3)
 * / V (OutputVars::CalcAndConvert, src/OutputVars.cpp:129-180). */
int gb_virial(gb_box *box, double *out16);
/* SingleMoleculeInter (src/CalculateEnergy.cpp:1494-1556): real-space
 * energy of molecule `mol` at its current position with its neighbourhood,
 * at two coupling pairs.  lambdas4 = old VDW, new VDW, old Coulomb, new
 * Coulomb; out4 = old inter, old real, new inter, new real (K). */
int gb_single_molecule_inter(gb_box *box, int32_t mol, const double *lambdas4,
                             double *out4);
/* ParticleInter (src/CalculateEnergy.cpp:727-785): atom `part` of molecule
 * `mol` (its kind and charge) at each of ntrials positions (1..256), LJ and
 * real-space energies and the RcutLow overlap flag against every atom in the
 * cell list.  As in the reference nothing is excluded: a CBMC caller takes
 * the molecule out of the cell list first (gb_cell_remove_mol, as
 * MoleculeTransfer::Transform does, src/moves/MoleculeTransfer.h:100-106). */
int gb_particle_inter(gb_box *box, int32_t mol, int32_t part,
                      const double *trials, int32_t ntrials, double *en,
                      double *real, int32_t *overlap);
/* BoxForce (src/CalculateEnergy.cpp:268-406): energies plus atom and
 * molecule forces (host arrays may be NULL). */
int gb_box_force(gb_box *box, double *inter, double *real, double *atom_force,
                 double *mol_force);
/* BoxForce(potential, coords, ...) of the given coordinates xyz [n_atoms * 3]
 * at the box's edges, as MultiParticle::CalcEn calls it on its trial
 * coordinates (src/moves/MultiParticle.h:424-428); the box's own state is
 * untouched. */
int gb_box_force_coords(gb_box *box, const double *xyz, double *inter,
                        double *real, double *atom_force, double *mol_force);
/* BoxInter(potential, coords, boxAxes, box) (src/CalculateEnergy.cpp:
 * 157-266) of coordinates xyz [n_atoms * 3] at edges edges3[3], on a cell
 * grid of those edges built for the call (VolumeTransfer::CalcEn,
 * src/moves/VolumeTransfer.h:150-178); the box's own state is untouched. */
int gb_box_inter_coords(gb_box *box, const double *edges3, const double *xyz,
                        double *inter, double *real);
/* CalculateTorque (src/CalculateEnergy.cpp:1365-1406) from the forces of the
 * last gb_box_force and gb_box_force_reciprocal calls. */
int gb_calculate_torque(gb_box *box, double *mol_torque);

/* ---- Ewald (src/Ewald.h:46-228) ---- */
int gb_num_kvectors(gb_box *box, int32_t *k_count, int32_t *kmax);
/* k-vector tables and Ref sums: kx, ky, kz, prefact, hsqr, sumRref, sumIref,
 * seven arrays of k_count doubles (Ewald::RecipInitOrth,
 * src/Ewald.cpp:847-903) */
int gb_get_kvectors(gb_box *box, double *out7);
int gb_get_sums_new(gb_box *box, double *sum_r, double *sum_i);
/* BoxReciprocalSetup (src/Ewald.cpp:193-274) + SetRecipRef (:1021-1053) */
int gb_box_reciprocal_setup(gb_box *box);
/* BoxReciprocalSums (src/Ewald.cpp:281-361) for the current coordinates */
int gb_box_reciprocal_sums(gb_box *box);
/* BoxReciprocalSums(box, molCoords) (src/Ewald.cpp:281-361): the New sums of
 * the given coordinates xyz [n_atoms * 3] with the current (Ref) k-vector
 * set, as MultiParticle::CalcEn calls it on its trial coordinates
 * (src/moves/MultiParticle.h:424-431). */
int gb_box_reciprocal_sums_coords(gb_box *box, const double *xyz);
/* BoxReciprocal(box, isNewVolume) (src/Ewald.cpp:375-406): the energy of the
 * New sums with the prefactors of the New k-vector set (is_new_volume = 1,
 * after gb_recip_init for trial edges) or of the current Ref set (0). */
int gb_box_reciprocal(gb_box *box, int32_t is_new_volume, double *energy);
/* RecipInit(box, boxAxes) (src/Ewald.cpp:835-903) for trial edges
 * edges3[3]: builds the New k-vector set (imageSize, kx/ky/kz, hsqr,
 * prefact); k_count (may be NULL) receives its size.  The current set is
 * untouched. */
int gb_recip_init(gb_box *box, const double *edges3, int32_t *k_count);
/* BoxReciprocalSetup(box, molCoords) (src/Ewald.cpp:193-274): the New sums
 * of coordinates xyz [n_atoms * 3] with the New k-vector set, the coordinates
 * lying inside the edges that set was built for (VolumeTransfer::CalcEn,
 * src/moves/VolumeTransfer.h:160-176). */
int gb_box_reciprocal_setup_coords(gb_box *box, const double *xyz);
/* UpdateRecipVec (src/Ewald.cpp:1462-1487): swap the New and Ref k-vector
 * sets.  Until gb_set_box gives the box the edges of its new Ref set, only
 * gb_set_box, gb_recip_init, gb_box_reciprocal, gb_box_reciprocal_setup_coords,
 * gb_box_inter_coords, gb_box_edges and the energy accessors are valid
 * (others return GB_ERR_STATE).  Not for a box with a Monte Carlo loop. */
int gb_update_recip_vec(gb_box *box);
/* MolReciprocal (src/Ewald.cpp:409-473): fills the New sums, returns the
 * energy difference against the running reciprocal energy */
int gb_mol_reciprocal(gb_box *box, int32_t mol, const double *new_pos,
                      double *delta);
/* SwapDestRecip / SwapSourceRecip (src/Ewald.cpp:478-531, 657-710) */
int gb_swap_dest_recip(gb_box *box, int32_t mol, const double *pos,
                       double *delta);
int gb_swap_source_recip(gb_box *box, int32_t mol, const double *pos,
                         double *delta);
int gb_update_recip(gb_box *box);   /* UpdateRecip, src/Ewald.cpp:1420-1434 */
int gb_copy_recip(gb_box *box);     /* CopyRecip, src/Ewald.cpp:1441-1460 */
int gb_box_self(gb_box *box, double *self); /* BoxSelf :1125-1163 */
int gb_mol_correction(gb_box *box, int32_t mol, double *corr); /* :1056-1085 */
/* SwapSelf (src/Ewald.cpp:1375-1391): self energy of molecule `mol`;
 * SwapCorrection (src/Ewald.cpp:1311-1333): its intramolecular correction at
 * positions pos [n_atoms_of_mol * 3] in this box (MoleculeTransfer::CalcEn,
 * src/moves/MoleculeTransfer.h:112-128). */
int gb_swap_self(gb_box *box, int32_t mol, double *self);
int gb_swap_correction(gb_box *box, int32_t mol, const double *pos,
                       double *corr);
/* BoxForceReciprocal (src/Ewald.cpp:1496-1596) from the New sums */
int gb_box_force_reciprocal(gb_box *box, double *atom_force_rec,
                            double *mol_force_rec);

/* ---- CellList (src/CellList.h:22-86) ---- */
int gb_grid_all(gb_box *box);  /* GridAll, src/CellList.cpp:220-237 */
/* RemoveMol / AddMol (src/CellList.cpp:81-135): take molecule `mol` out of
 * the cell list, or put it back at its current coordinates.  While any
 * molecule is out, the Monte Carlo and checkpoint calls return GB_ERR_STATE;
 * gb_grid_all puts every molecule back. */
int gb_cell_remove_mol(gb_box *box, int32_t mol);
int gb_cell_add_mol(gb_box *box, int32_t mol);
/* cell index of every atom (GetCellListNeighbor's mapParticleToCell,
 * src/CellList.cpp:258-285) and the cells per edge */
int gb_cell_membership(gb_box *box, int32_t *cell_of_atom, int32_t *edge3);

/* ---- state ---- */
int gb_box_edges(gb_box *box, double *edges3);  /* BoxDimensions axes */
/* New box edges edges3[3] with coordinates xyz [n_atoms * 3] (inside them)
 * and centres com [n_mol * 3] (may be NULL: computed as COM::CalcCOM does):
 * what VolumeTransfer::Accept leaves after an accepted move
 * (src/moves/VolumeTransfer.h:241-270: coordinates, BoxDimensions,
 * UpdateRecip, UpdateRecipVec), with the derived state rebuilt as
 * System::Init does: CellList::ResizeGrid + GridAll (src/CellList.cpp:
 * 138-237), the k-vector set of the edges (the one gb_recip_init built for
 * them, else a new one), the structure factors and the running energies.
 * Not for a box with a Monte Carlo loop (GB_ERR_STATE). */
int gb_set_box(gb_box *box, const double *edges3, const double *xyz,
               const double *com);
int gb_get_coords(gb_box *box, double *xyz, double *com);
/* Replace the coordinates [n_atoms * 3] (inside the box) and molecule
 * centres [n_mol * 3] and bring every derived quantity in line, as
 * System::Init does after reading coordinates (src/System.cpp:67-100):
 * CellList::GridAll, the Ewald structure factors (BoxReciprocalSetup +
 * SetRecipRef) and the running energies (SystemTotal).  com may be NULL: the
 * centres are then computed as COM::CalcCOM does (src/COM.h:47-68), which
 * re-wraps each molecule's atoms.  The Monte Carlo state (step, move
 * settings) is kept; the next gb_mc_run scores moves against the new
 * state. */
int gb_set_coords(gb_box *box, const double *xyz, const double *com);
/* running energies inter, real, recip, self, correction (SystemPotential) */
int gb_get_energy(gb_box *box, double *e5);
int gb_set_energy(gb_box *box, const double *e5);

/* ---- device-resident Monte Carlo loop ----
 * System::ChooseAndRunMove / RunMove (src/System.cpp:262-302) with the
 * Translate, Rotate and MultiParticle moves (src/moves/Translate.h,
 * Rotation.h, MultiParticle.h) and MoveSettings adjustment
 * (src/MoveSettings.cpp:157-265).  Proposals come from the reference's
 * MT19937 stream seeded with Random_Seed (src/PRNGSetup.h:28) and the
 * MultiParticle move from Philox4x64-10 keyed (step, seed). */
typedef struct gb_mc_params {
  uint32_t seed;          /* Random_Seed */
  double frac[3];         /* DisFreq, RotFreq, MultiParticleFreq */
  int32_t adj_steps;      /* AdjSteps */
  int32_t use_scales;     /* 1: start from scales[] instead of the defaults */
  double scales[4];       /* displacement, rotation, MP t_max, MP r_max */
  int32_t recompute_freq; /* GB300RecomputeFreq (mixed form), 0 = never */
  int32_t cluster_size;   /* mixed form: CTAs per chain, 2, 4, 8 or 16
                             (0 = the largest that fits) */
  int32_t flush_every;    /* not used (kept for layout): the mixed form's
                             structure factors are float-float and need no
                             periodic FP64 fold */
  int32_t move_buffer;    /* moves drawn and uploaded per chunk (0 = 65536) */
  int32_t unit_lanes;     /* mixed form: threads per real-space unit (one
                             atom's old or new position against one
                             neighbour cell's slots): 32, 64, 128 or 256
                             (0 = the smallest of 32, 64, 128 at least the
                             mean atoms per cell, else 128) */
  int32_t grid_ctas;      /* FP64 form: CTAs of the cooperative grid, 2 to
                             the SM count (0 = one per SM) */
  int32_t writer_kchunk;  /* FP64 form: 1 = the CTAs that write the next
                             move's context also hold k-vectors (the
                             k-chunk spreads over the whole grid); 0 = they
                             hold none when they are at most half the grid */
  int32_t moves_in_flight; /* FP64 form: 2 = the next move runs while this
                              one is decided, on both of its outcomes, and
                              one CTA of the grid only decides; 1 = one move
                              at a time (0 = 2 where the grid has a CTA to
                              spare for deciding, else 1) */
} gb_mc_params;

int gb_mc_init(gb_box *box, const gb_mc_params *params);
/* Run steps [first_step, first_step + nsteps).  Trace arrays may be NULL;
 * otherwise each has nsteps entries (de: 3 per step). */
int gb_mc_run(gb_box *box, int64_t first_step, int64_t nsteps, int32_t *kind,
              int32_t *mol, int32_t *accepted, double *de);
/* scales4: displacement, rotation, MP t_max, MP r_max;
 * counts6: tries/accepted for displacement, rotation, MultiParticle */
int gb_mc_state(gb_box *box, double *scales4, int64_t *counts6);

/* Device time spent in this box's Monte Carlo kernels since the last reset,
 * measured with CUDA events on the box's stream: chain kernels (translate /
 * rotate segments) and MultiParticle kernel sequences.  No reference
 * counterpart (measurement). */
int gb_mc_timing(gb_box *box, int32_t reset, double *chain_ms,
                 int64_t *chain_launches, int64_t *chain_moves, double *mp_ms,
                 int64_t *mp_moves);
/* Polls after which a wait inside the FP64 chain kernel (the grid barrier,
 * the partials, the next move's context, the decision word) gives up, 0 for
 * the default 2^22 (seconds of waiting).  A wait that gives up sets the
 * box's device error word: the CTAs leave the kernel without committing the
 * move, gb_mc_run returns GB_ERR_TIMEOUT, and the coordinates, energies and
 * structure factors stay as they were before the call; gb_mc_init clears
 * the error before the loop runs again.  No reference counterpart (the
 * reference has no device-side waits). */
int gb_mc_set_wait_limit(gb_box *box, int64_t polls);
/* Where the device time of the FP64 chain goes (no reference counterpart):
 * the clocks of a work CTA and of the deciding CTA (the last) since the
 * last call, per phase of a move (loading the move's context, listing the
 * real-space pairs, pair terms and k-vectors to the partials, waiting for
 * the decision, commit and the next context), as us13[0..9] (the work
 * CTA's five, then the last CTA's five) in microseconds at the rated SM
 * clock.  The work CTA is CTA 0 with one move in flight and the first CTA
 * with a k-chunk with two (the deciding CTA then only waits for the
 * partials, decides and commits: its listing phase is zero).  With one
 * move in flight us13[10] and [11]: when, counted from the end of its own
 * phase A, the last CTA had every partial and every flag of the next
 * context, and us13[12] when CTA 0 had written its part of the next
 * context (zero with two moves in flight); and the moves each CTA timed.
 * `enable` switches the collection on or off for the following runs.  The
 * mixed form is not timed here. */
int gb_mc_profile(gb_box *box, int32_t enable, double *us13, int64_t *moves2);
/* Mixed form: relative difference between the running energies and the
 * periodic full FP64 recompute (inter, real, recip, total), largest and
 * latest, and the number of recomputes so far.  No reference counterpart
 * (the reference's check is Simulation::RecalculateAndCheck,
 * src/Simulation.cpp:170-223, at 1e-3). */
int gb_mc_drift(gb_box *box, double *max4, double *last4, int64_t *recomputes);
/* Launch geometry gb_mc_init chose for this box's chain kernel: CTAs that
 * run one chain (the thread-block cluster size of the mixed form, the
 * cooperative grid of the FP64 form), how many such chains the GPU holds at
 * once, and the dynamic shared memory per CTA (mixed form).  No reference
 * counterpart. */
int gb_mc_layout(gb_box *box, int32_t *ctas_per_chain, int32_t *max_concurrent,
                 int64_t *smem_bytes);
/* One launch shape of a chain and its trial time (gb_mc_autotune). */
typedef struct gb_mc_shape {
  int32_t ctas;           /* mixed form: cluster size; FP64 form: grid CTAs */
  int32_t unit_lanes;     /* mixed form: threads per real-space unit */
  int32_t writer_kchunk;  /* FP64 form: context writers hold k-vectors */
  int32_t moves_in_flight;/* FP64 form: 1 or 2 */
  int32_t max_concurrent; /* chains of this shape the GPU holds at once */
  double us_per_move;     /* trial latency (0: the shape does not fit) */
} gb_mc_shape;
/* Autotuner of the chain geometry (no reference counterpart).  Mixed form:
 * the cluster size (2, 4, 8, 16: the k-chunk each CTA holds and the CTAs on
 * one move) times the threads per real-space unit (32, 64, 128: how a
 * neighbour cell's slots are tiled over threads).  FP64 form: the grid's
 * CTAs (the SM count and 3/4, 1/2, 1/4 of it: the threads on one move and
 * the k-chunk per CTA) times whether the context writers hold k-vectors
 * (the k-chunk at a fixed grid) times one or two moves in flight.  Each shape that fits the box runs a trial
 * segment of `trial_moves` moves (0 = 200) on the box's own state, which is
 * checkpointed and restored around every trial; the best shape for the
 * objective is kept: 0 = shortest move latency of one chain, 1 = most
 * moves/s with as many chains as the GPU holds at once (mixed form; the
 * FP64 form holds one chain).  The Monte Carlo state after the call is the
 * state before it.  `chosen` (may be NULL) receives the kept shape; `tried`
 * (may be NULL) up to `cap` shapes in the order tried, their number in
 * *n_tried (may be NULL). */
int gb_mc_autotune(gb_box *box, int32_t objective, int32_t trial_moves,
                   gb_mc_shape *chosen, gb_mc_shape *tried, int32_t cap,
                   int32_t *n_tried);
/* The launch shape gb_mc_init (or the autotuner) chose for this box's
 * chain, its trial time zero.  No reference counterpart. */
int gb_mc_shape_get(gb_box *box, gb_mc_shape *shape);
/* The CUDA stream (cudaStream_t) every call on this machine is ordered on. */
int gb_box_stream(gb_box *box, void **stream);

/* Run the same number of steps on several boxes concurrently (one launch
 * for all single-molecule segments).  Each box must have gb_mc_init. */
int gb_mc_run_batch(gb_box **boxes, int32_t nboxes, int64_t first_step,
                    int64_t nsteps);

/* ---- Checkpoints ----
 * The role of the reference's Checkpoint (src/Checkpoint.h:27-120) in a
 * format of this library's own: a run that loads a checkpoint continues with
 * the same moves, decisions and coordinates, bit for bit, as a run that
 * never stopped (the reference's restart tests pin the same property,
 * test/src/CheckpointTest.cpp).  Saved: coordinates, molecule centres, the
 * cell grid's slot order, the FP64 structure factors, the running energies
 * and, after gb_mc_init, the step, the MT19937 state of the move stream,
 * the move settings and the drift records.  A checkpoint loads into a box
 * created from the same system and configuration (and gb_mc_init'ed first
 * when it holds Monte Carlo state); anything else is GB_ERR_ARG /
 * GB_ERR_STATE. */
int gb_checkpoint_size(gb_box *box, int64_t *bytes);
int gb_checkpoint_save(gb_box *box, void *buf, int64_t bytes);
int gb_checkpoint_load(gb_box *box, const void *buf, int64_t bytes);

/* ---- The reference's checkpoint file (src/Checkpoint.h:27-169) ----
 * GOMC checkpoints (CheckpointOutput::saveCheckpointFile,
 * src/CheckpointOutput.cpp:55-90, a cereal binary archive) carry the Monte
 * Carlo loop state -- step, the MT19937 state (src/MersenneTwister.h
 * save / load), the move settings (src/MoveSettings.h) -- followed by the
 * molecule lookup, the molecule setup and the PDB atom records.  These
 * calls exchange the loop state with a stock GOMC run: read it from a GOMC
 * checkpoint into gb_gomc_chk, move it into or out of a box's loop, and
 * write a GOMC checkpoint as a copy of a template checkpoint of the same
 * system (the reference's own, which holds the records a box does not) with
 * the loop state replaced.  Coordinates travel separately (gb_set_coords /
 * gb_get_coords; the reference restarts them from its restart coordinate
 * files).  Per-move arrays hold molecule kind 0 (the loop moves one kind). */
#define GB_CHK_BOXES 2
#define GB_CHK_MOVES 16
#define GB_CHK_MP 2
typedef struct gb_gomc_chk {
  uint64_t step, true_step;   /* stepNumber, trueStepNumber */
  uint32_t mt_state[624];     /* saveArray[0..623] */
  uint32_t mt_left;           /* saveArray[624] */
  uint32_t seed_location, seed_left, seed_value;
  int32_t n_box, n_move, n_kind;  /* the file's vector shapes */
  double scale[GB_CHK_BOXES][GB_CHK_MOVES];
  double accept_percent[GB_CHK_BOXES][GB_CHK_MOVES];
  uint32_t accepted[GB_CHK_BOXES][GB_CHK_MOVES];
  uint32_t tries[GB_CHK_BOXES][GB_CHK_MOVES];
  uint32_t temp_accepted[GB_CHK_BOXES][GB_CHK_MOVES];
  uint32_t temp_tries[GB_CHK_BOXES][GB_CHK_MOVES];
  uint32_t mp_tries[GB_CHK_BOXES][GB_CHK_MP];     /* MPDISPLACE, MPROTATE */
  uint32_t mp_accepted[GB_CHK_BOXES][GB_CHK_MP];
  uint32_t mp_interval_accepted[GB_CHK_BOXES][GB_CHK_MP];
  uint32_t mp_interval_tries[GB_CHK_BOXES][GB_CHK_MP];
  double mp_t_max[GB_CHK_BOXES], mp_r_max[GB_CHK_BOXES];
  int32_t single_move_accepted[GB_CHK_BOXES];
  int64_t records_offset;     /* bytes before the lookup / setup records */
} gb_gomc_chk;
/* CheckpointSetup::loadCheckpointFile's reading of the loop state
 * (src/CheckpointSetup.cpp:45-82, SetMoveSettings / SetPRNGVariables
 * :118-148).  GB_ERR_ARG for a truncated or malformed archive. */
int gb_gomc_checkpoint_read(const void *buf, int64_t bytes, gb_gomc_chk *out);
/* A GOMC checkpoint: `tmpl` (a GOMC checkpoint of the same system) with the
 * loop state of `in`; *out_bytes receives the size (out == NULL: size
 * only; GB_ERR_ARG when it exceeds out_cap). */
int gb_gomc_checkpoint_write(const void *tmpl, int64_t tmpl_bytes,
                             const gb_gomc_chk *in, void *out,
                             int64_t out_cap, int64_t *out_bytes);
/* The box's loop state as a GOMC checkpoint holds it (box 0, kind 0), and
 * back: after gb_mc_set_gomc_state the next gb_mc_run starts at chk->step
 * with the reference's random stream and move settings at that step. */
int gb_mc_get_gomc_state(gb_box *box, gb_gomc_chk *out);
int gb_mc_set_gomc_state(gb_box *box, const gb_gomc_chk *in);

/* ---- Continuous-batching job server ----
 * No counterpart in the reference (it runs one simulation per process,
 * src/Simulation.cpp:116-168).  A server runs many independent
 * mixed-precision NVT jobs (translate / rotate moves) on one GPU.  Each
 * round launches the next segment of every resident job (at most `quantum`
 * moves, one launch per cluster size, launches overlapping on the device),
 * admits queued jobs first come first served while their estimated device
 * memory fits `mem_budget` and their chains fit the GPU's free CTA slots,
 * and retires finished jobs (their final coordinates and running energies
 * are kept on the host).  A job's results do not depend on which other jobs
 * share its rounds.  Rounds run either on the caller's thread
 * (gb_server_step) or on a worker thread (gb_server_start .. gb_server_drain);
 * gb_server_submit may be called from any thread at any time. */
typedef struct gb_server gb_server;
enum gb_job_status {
  GB_JOB_QUEUED = 0,
  GB_JOB_RUNNING = 1,
  GB_JOB_DONE = 2,
  GB_JOB_FAILED = 3
};
typedef struct gb_server_config {
  int32_t device;
  int32_t quantum;       /* moves per round of a job with 4,096 k-vectors per
                            CTA (0 = 1000); a job's own quantum scales
                            inversely with its time per move, modelled as
                            2,560 + its k-vectors per CTA, within
                            [quantum/4, 8 quantum] */
  int64_t mem_budget;    /* device bytes for job state (0 = 90% of free) */
  int32_t max_resident;  /* at most this many resident jobs (0 = no cap) */
} gb_server_config;
int gb_server_create(const gb_server_config *cfg, gb_server **out);
/* Stops the worker after its current round; drops queued and resident jobs. */
void gb_server_destroy(gb_server *srv);
/* Queue a job of `nsteps` moves; the inputs are copied.  cfg->precision must
 * be GB_MIXED, mc->frac[2] (MultiParticle) 0; mc->cluster_size 0 lets the
 * server pick the cluster from the job's k-vector count.  `sweep_moves` (0 =
 * molecules of the job) defines a sweep for the latency statistics. */
int gb_server_submit(gb_server *srv, const gb_system_desc *sys,
                     const gb_config *cfg, const gb_mc_params *mc,
                     int64_t nsteps, int64_t sweep_moves, int64_t *job_id);
/* The device bytes the server would reserve for such a job at admission
 * (its memory estimate) and the CTAs per chain it would give it. */
int gb_server_estimate(gb_server *srv, const gb_system_desc *sys,
                       const gb_config *cfg, const gb_mc_params *mc,
                       int64_t *bytes, int32_t *ctas_per_chain);
/* One round on the calling thread (GB_ERR_STATE while a worker runs);
 * *pending = jobs queued or resident afterwards. */
int gb_server_step(gb_server *srv, int32_t *pending);
/* Run rounds on a worker thread until gb_server_drain. */
int gb_server_start(gb_server *srv);
/* Wait until every submitted job has finished (or failed), then stop the
 * worker.  timeout_s <= 0 waits without limit; GB_ERR_TIMEOUT otherwise. */
int gb_server_drain(gb_server *srv, double timeout_s);
/* status (gb_job_status), moves done, and times (s since server creation)
 * of submission, admission and completion */
int gb_server_job(gb_server *srv, int64_t job, int32_t *status,
                  int64_t *steps_done, double *times3);
/* Final coordinates [n_atoms * 3], molecule centres [n_mol * 3] and running
 * energies (inter, real, recip, self, correction) of a finished job. */
int gb_server_result(gb_server *srv, int64_t job, double *xyz, double *com,
                     double *energy5);
/* out12: jobs done, moves run, wall seconds from the first admission to the
 * last completion, moves/s over that span, per-sweep latency p50 and p99
 * (ms), job latency (submission to completion) p50 and p99 (s), rounds, mean
 * resident jobs per round, helper-thread seconds (summed over the helper
 * threads) spent on set-ups and FP64 recomputes, seconds spent in rounds
 * (launch to completion). */
int gb_server_stats(gb_server *srv, double *out12);
/* out10: means over the rounds so far, taken after each round's admission,
 * of the jobs admitted (set up, running or recomputing), the jobs in the
 * round's launches, the fraction of the GPU's chain CTA slots held (two per
 * SM), the fraction of the GPU's shared memory held and the jobs still
 * queued; then how many admission passes stopped at the queue's head for
 * want of device memory, of shared memory, of CTA slots; then the mean
 * launch balance of a round (its launches' device time weighted by their
 * CTAs, over its longest launch's time those CTAs were held: 1 = every chain
 * ran until the round's end) and the seconds of round wall time outside
 * each round's longest launch. */
int gb_server_occupancy(gb_server *srv, double *out10);
const char *gb_server_error(const gb_server *srv);

/* ---- Gibbs ensemble (GEMC NVT) of single-site LJ particles ----
 * Two boxes exchanging volume and molecules, run on one GPU as one
 * persistent launch of one thread-block cluster: the reference's GEMC move
 * loop (System::ChooseAndRunMove / RunMove, src/System.cpp:262-302) over
 * Translate (src/moves/Translate.h:52-138), MoleculeTransfer with CBMC
 * first-atom trials (src/moves/MoleculeTransfer.h:71-245,
 * src/cbmc/DCSingle.cpp:23-90) and VolumeTransfer GEMC-NVT
 * (src/moves/VolumeTransfer.h:71-318), with the MoveSettings adjustment
 * (src/MoveSettings.cpp:94-238) and the reference's MT19937 stream seeded
 * with Random_Seed (drawn on the device, since how many numbers a move takes
 * depends on the molecule counts of the boxes).  One molecule kind of one
 * LJ (Mie) site, no charges, no tail correction; both boxes must fit one
 * CTA's shared memory (about 2,900 molecules in all in the mixed form, 3,300
 * in the FP64 form: GB_ERR_UNSUPPORTED beyond). */
typedef struct gb_gemc gb_gemc;
typedef struct gb_gemc_desc {
  int32_t n0, n1;               /* molecules in box 0 and box 1 */
  const double *pos0, *pos1;    /* [n0 * 3], [n1 * 3] as read from the PDBs */
  double box0[3], box1[3];      /* orthogonal edges, A */
  double epsilon, sigma, n_mie; /* the LJ site: K, A, repulsion exponent */
} gb_gemc_desc;
typedef struct gb_gemc_config {
  double temperature, rcut, rcut_low; /* Temperature, Rcut, RcutLow */
  double frac[3];         /* DisFreq, VolFreq, SwapFreq */
  int32_t adj_steps;      /* AdjSteps */
  int32_t cbmc_first;     /* CBMC_First (1..16) */
  int32_t precision;      /* GB_FP64, or GB_MIXED: FP32 pair energies on
                             exact fixed-point separations, FP64 sums */
  int32_t device;
  int32_t cluster_size;   /* CTAs of the cluster: 1, 2, 4, 8, 16 (0 = 16) */
  uint32_t seed;          /* Random_Seed */
} gb_gemc_config;
/* System::Init of the two boxes: wrapped coordinates, centres, the molecule
 * lookup (box 0's molecules then box 1's), initial SystemTotal. */
int gb_gemc_create(const gb_gemc_desc *desc, const gb_gemc_config *cfg,
                   gb_gemc **out);
void gb_gemc_destroy(gb_gemc *g);
const char *gb_gemc_error(const gb_gemc *g); /* NULL: last create error */
/* Steps [first_step, first_step + nsteps), continuing the last run.  Trace
 * arrays may be NULL; per step trace_i5 = move kind (0 displacement, 10
 * molecule transfer, 13 volume exchange: src/MoveConst.h), box (source box
 * of a transfer, first box of a volume pair), molecule (-1 if none), accepted,
 * molecules in box 0 after the step; trace_d8 = four move values
 * (displacement: dE, overlap; transfer: new and old Rosenbluth weights, new
 * and old trial energies; volume: the trial energies of both boxes), then
 * the running energies and volumes of both boxes.  GB_ERR_STATE if a volume
 * exchange would shrink a box below 2 Rcut (the reference exits there). */
int gb_gemc_run(gb_gemc *g, int64_t first_step, int64_t nsteps,
                int32_t *trace_i5, double *trace_d8);
/* running inter energies, edges of both boxes, molecules in box 0, move
 * scales (displacement, volume; per box), tries / accepted of displacement,
 * transfer and volume per box, device time of the last run (ms) */
int gb_gemc_state(gb_gemc *g, double *energy2, double *edges6,
                  int32_t *n_box0, double *scales4, int64_t *counts12,
                  double *last_ms);
/* coordinates and centres of every molecule [n * 3] and the molecule
 * lookup [n] (box 0's section first) */
int gb_gemc_coords(gb_gemc *g, double *xyz, double *com, int32_t *lookup);
/* full FP64 recompute of both boxes' inter energies (CalculateEnergy::
 * SystemTotal, src/CalculateEnergy.cpp:83-153) */
int gb_gemc_system_total(gb_gemc *g, double *energy2);
/* Where the device time of the move loop goes (no reference counterpart):
 * the clocks of the cluster's first CTA since the last call, per move kind
 * (displacement, transfer, volume) and phase (drawing the random numbers,
 * pair energies, exchange of the partials, decision, commit), as us15 in
 * microseconds at the rated SM clock, and the moves of each kind; `enable`
 * switches the collection on or off for the following runs. */
int gb_gemc_profile(gb_gemc *g, int32_t enable, double *us15,
                    int64_t *moves3);

/* ---- Reciprocal energy without device allocation ----
 * No counterpart in the reference.  It is the reduction behind BoxReciprocal
 * (src/Ewald.cpp:375-406), E = sum_k prefact[k] (sumR[k]^2 + sumI[k]^2),
 * over caller-owned device arrays of K doubles, with the result written to
 * the device double *d_energy, ordered on `stream` (a cudaStream_t; NULL is
 * the legacy default stream) of the current device.
 *
 * For callers that may not allocate device memory once running: a serving
 * loop that admits jobs by device memory and has committed all of it, or a
 * host whose device memory belongs to another allocator.  The call issues no
 * cudaMalloc/cudaFree and no allocating library routine; its scratch is a
 * fixed 8 KiB device array inside this library, one FP64 partial per 256
 * k-vectors, hence the limit on K (larger K: GB_ERR_CAPACITY, nothing
 * launched).  The first call on a device looks up that array's address with
 * the device current and keeps it for the life of the process; make it
 * before any stream capture, and do not call this entry point again on a
 * device after cudaDeviceReset there (the kept address belonged to the
 * context the reset destroyed).  Calls that overlap
 * in time on one device share the array and race: serialise them.  The sum
 * is taken in the order of gb_box_reciprocal.  Errors: GB_ERR_ARG (null
 * pointer, K < 0), GB_ERR_CAPACITY, GB_ERR_CUDA; gb_last_error(NULL) gives
 * the message. */
#define GB_RECIP_NOALLOC_MAX_PARTIALS 1024
#define GB_RECIP_NOALLOC_MAX_K (256 * GB_RECIP_NOALLOC_MAX_PARTIALS)
int gb_recip_energy_noalloc(const double *d_sumR, const double *d_sumI,
                            const double *d_prefact, int32_t K,
                            double *d_energy, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* GOMC_GB300_H */
