/* CPU oracle for the GOMC Monte Carlo energy path -- TEST INFRASTRUCTURE.
 *
 * A plain-C restatement of the reference algorithms (GOMC 2.80) for one
 * orthogonal NVT box: cell list, Lennard-Jones (Mie) + erfc-screened Coulomb
 * under the minimum image, Ewald k-vectors / structure factors / molecule and
 * insert/delete deltas, self and intramolecular correction terms, box forces,
 * reciprocal forces and torques, the Mersenne-Twister driven translate/rotate
 * moves, the Philox-driven MultiParticle move and move-size adjustment.
 * Every function cites the reference lines it follows.
 *
 * Only tests, the smoke check and the CPU-baseline leg of the benchmark use
 * this library, and only as the checker; the product path never links it.
 */
#ifndef GOMC_ORACLE_H
#define GOMC_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ora_sys ora_sys;

/* Build a box the way System::Init does (src/System.cpp:67-100): wrap every
 * atom into the box (Coordinates::WrapCoordinate), compute molecule centres
 * (COM::CalcCOM, src/COM.h:47-68), grid the cell list, set up the Ewald
 * k-vectors and structure factors and the initial SystemTotal energies. */
ora_sys *ora_create(int n_atoms, int n_mol, const double *pos,
                    const int *kind, const double *charge,
                    const int *mol_start, int n_kinds, const double *eps,
                    const double *sigma, const double *nexp,
                    const double *box, double rcut, double rcut_low,
                    double rcut_coul, double tolerance, int ewald,
                    int electrostatic, double temperature);
void ora_destroy(ora_sys *s);
void ora_set_threads(int n);

int ora_num_k(const ora_sys *s);
int ora_num_cells(const ora_sys *s);
void ora_get_coords(const ora_sys *s, double *xyz);
void ora_get_com(const ora_sys *s, double *xyz);
void ora_set_coords(ora_sys *s, const double *xyz, const double *com);
/* kx, ky, kz, prefact, hsqr, sumRref, sumIref: 7 arrays of length K */
void ora_get_kvec(const ora_sys *s, double *out7);
void ora_get_sum_new(const ora_sys *s, double *sr, double *si);
/* cell index of every atom, plus edge counts */
void ora_get_cells(const ora_sys *s, int *cell_of_atom, int *edge3);
/* running energies: inter, real, recip, self, correction */
void ora_get_energy(const ora_sys *s, double *e5);
void ora_set_energy(ora_sys *s, const double *e5);

/* Full recompute (CalculateEnergy::SystemTotal + UpdateVectorsAndRecipTerms)
 * out9: inter real recip self correction tail intraBond intraNonbond total */
void ora_system_total(ora_sys *s, double *out9);
void ora_grid_all(ora_sys *s);

/* Soft-core settings of FFParticle at lambda < 1 (Forcefield sc_alpha,
 * sc_sigma_6, sc_power, sc_coul; src/Forcefield.cpp:59-75). */
typedef struct ora_softcore {
  double alpha, sigma6;
  int power, coul;
} ora_softcore;
/* CalculateEnergy::SingleMoleculeInter (src/CalculateEnergy.cpp:1494-1556):
 * lam = old VDW, new VDW, old Coulomb, new Coulomb lambdas;
 * out = old inter, old real, new inter, new real. */
void ora_single_molecule_inter(const ora_sys *s, int m, const double *lam,
                               const ora_softcore *sc, double *out);
/* CalculateEnergy::VirialCalc + Ewald::VirialReciprocal
 * (src/CalculateEnergy.cpp:411-579, src/Ewald.cpp:1168-1305), LRC off.
 * out16 = inter, real, recip, total, diagonals of interTens, realTens,
 * recipTens, totalTens. */
void ora_virial(ora_sys *s, double *out16);
/* CalculateEnergy::MoleculeInter with the molecule removed from the cell list
 * first (as Translate::CalcEn does).  Returns overlap. */
int ora_molecule_inter(ora_sys *s, int m, const double *newpos, double *dlj,
                       double *dreal);
/* CalculateEnergy::ParticleInter for one trial position of atom `part` of
 * molecule m against the atoms in the cell list (src/CalculateEnergy.cpp:
 * 727-785); nothing is excluded, as in the reference. */
int ora_particle_inter(const ora_sys *s, int m, int part, const double *trial,
                       double *en, double *real);
/* CellList::RemoveMol / AddMol (src/CellList.cpp:81-135) */
void ora_cell_remove_mol(ora_sys *s, int m);
void ora_cell_add_mol(ora_sys *s, int m);
double ora_mol_reciprocal(ora_sys *s, const double *newpos, int m);
double ora_swap_dest_recip(ora_sys *s, const double *newpos, int m);
double ora_swap_source_recip(ora_sys *s, const double *oldpos, int m);
void ora_update_recip(ora_sys *s);
void ora_copy_recip(ora_sys *s);
double ora_box_self(const ora_sys *s);
double ora_mol_correction(const ora_sys *s, int m);
/* BoxForce on coords (NULL = current): atom forces aF[N*3], molecule forces
 * mF[M*3]; returns inter and real energies */
void ora_box_force(ora_sys *s, const double *coords, double *aF, double *mF,
                   double *inter, double *real);
/* BoxReciprocalSums on coords (NULL = current) into sumRnew/sumInew and the
 * returned energy (BoxReciprocal with isNewVolume=false) */
double ora_box_reciprocal_sums(ora_sys *s, const double *coords);
void ora_box_force_recip(ora_sys *s, const double *coords, double *aR,
                         double *mR);
void ora_torque(const ora_sys *s, const double *coords, const double *com,
                const double *aF, const double *aR, double *tq);

/* Mersenne Twister MT19937 and Philox4x64-10 streams */
typedef struct ora_mt ora_mt;
ora_mt *ora_mt_create(uint32_t seed);
void ora_mt_destroy(ora_mt *g);
uint32_t ora_mt_u32(ora_mt *g);
void ora_philox4x64(uint64_t c0, uint64_t c1, uint64_t c2, uint64_t c3,
                    uint64_t k0, uint64_t k1, uint64_t *out4);
double ora_u01_64(uint64_t v);
double ora_uneg11_64(uint64_t v);

/* Monte Carlo NVT loop over translate / rotate / MultiParticle moves. */
typedef struct ora_mc ora_mc;
ora_mc *ora_mc_create(ora_sys *s, uint32_t seed, const double *move_frac3,
                      int adj_steps);
void ora_mc_destroy(ora_mc *mc);
/* per step: kind, molecule (or MP type), accepted, overlap, dLJ, dReal, dRecip
 * (for MP: the new inter, real, recip) */
void ora_mc_run(ora_mc *mc, long first_step, long nsteps, int *kind, int *mol,
                int *acc, int *ovl, double *de3);
/* scales: disp, rot, mp_t_max, mp_r_max; counts: tries/accepted x 3 kinds */
void ora_mc_state(const ora_mc *mc, double *scales4, long *counts6);
void ora_mc_set_scales(ora_mc *mc, const double *scales4);

/* Gibbs ensemble (NVT) of single-site LJ particles in two boxes:
 * displacement, CBMC molecule transfer and volume exchange moves. */
typedef struct ora_gemc ora_gemc;
ora_gemc *ora_gemc_create(int n0, const double *pos0, int n1,
                          const double *pos1, const double *L0,
                          const double *L1, double eps, double sigma,
                          double nmie, double temperature, double rcut,
                          double rcut_low, uint32_t seed,
                          const double *frac3, int adj_steps, int ntrials);
void ora_gemc_destroy(ora_gemc *g);
/* frac3 = DisFreq, VolFreq, SwapFreq.  Per step: kind (0 displacement, 10
 * transfer, 13 volume), box, molecule, accepted, four move values and the
 * state after it (energies of both boxes, volumes, molecules in box 0).
 * Returns non-zero if a volume change would shrink a box below 2 Rcut. */
int ora_gemc_run(ora_gemc *g, long first, long nsteps, int *kind, int *box,
                 int *mol, int *acc, double *d4, double *state5);
void ora_gemc_get(const ora_gemc *g, double *xyz, double *com, int *lookup,
                  int *n0, double *e2, double *axes6);
void ora_gemc_system_total(const ora_gemc *g, double *e2);
void ora_gemc_settings(const ora_gemc *g, double *scale4, long *counts12);

#ifdef __cplusplus
}
#endif
#endif
