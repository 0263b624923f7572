// gb_box: one simulation box resident on one GPU, and the host-side set-up
// that mirrors System::Init (src/System.cpp:67-100).
#pragma once

#include "gb_internal.h"

#include <memory>
#include <string>
#include <vector>

namespace gb {

struct McState;  // Monte Carlo loop state (gb_mc.cu)

// One Ewald k-vector set (the kx/ky/kz/hsqr/prefact arrays and imageSize of
// src/Ewald.h:202-211) with the box edges it was built for.  A box keeps the
// current set (Ref) and a second one that RecipInit fills for trial edges
// (New); UpdateRecipVec swaps them (src/Ewald.cpp:1462-1487).
struct KSet {
  int K = 0, kmax = 0, nrun = 0;
  size_t cap = 0, run_cap = 0;  // allocated k-vectors, runs
  double L[3] = {0, 0, 0};
  double *kx = nullptr, *ky = nullptr, *kz = nullptr, *prefact = nullptr,
         *hsqr = nullptr;
  char4 *kn = nullptr;
  float *prefact_f = nullptr;
  int4 *krun = nullptr;
  int *krun_k = nullptr;
};

// Coordinates and cell grid of a trial state (other coordinates, other box
// edges) for the calls that take coordinates (BoxInter / BoxForce /
// BoxReciprocalSetup with newMolsPos in VolumeTransfer and MultiParticle).
struct TrialState {
  DevBox v{};                 // view: trial coordinates, grid, edges
  size_t cell_cap = 0;        // allocated ncell * cap
  size_t nbr_cap = 0;         // allocated ncell * 27
  std::vector<void *> allocs;
};

struct BoxConfig {
  double temperature = 298.0;
  double rcut = 9.0, rcut_low = 0.0, rcut_coulomb = 9.0, tolerance = 1e-5;
  int ewald = 1, electrostatic = 1;
  int precision = 0;  // 0 = FP64 plain form, 1 = mixed
  int device = 0;
  double sc_alpha = 0.0, sc_sigma = 0.0;  // soft-core settings
  int sc_power = 0, sc_coul = 0;
};

class Box {
 public:
  ~Box();
  static int Create(const HostSystem &sys, const BoxConfig &cfg, Box **out,
                    std::string *err);

  // ---- energy path (all run on `stream`) ----
  int GridAll();                                 // CellList::GridAll
  // CellList::ResizeGrid + GridAll on new box edges, coordinates, centres;
  // then the k-vector set of the edges, structure factors and running
  // energies as System::Init computes them
  int SetBox(const double L[3], const double *xyz, const double *com);
  int RecipInit(const double L[3]);              // Ewald::RecipInit -> New set
  int UpdateRecipVec();                          // Ewald::UpdateRecipVec
  // New sums of the given coordinates (host [N * 3]): with the New k-vector
  // set at its edges (BoxReciprocalSetup) or the Ref set (BoxReciprocalSums)
  int RecipSumsCoords(const double *xyz, bool new_set);
  int RecipEnergyNew(double *e, bool new_volume);  // Ewald::BoxReciprocal
  // BoxInter / BoxForce of given coordinates at given edges
  int BoxInterAt(const double L[3], const double *xyz, double *inter,
                 double *real);
  int BoxForceAt(const double *xyz, double *inter, double *real,
                 double *h_aF, double *h_mF);
  int SwapSelf(int m, double *e);                // Ewald::SwapSelf
  int SwapCorrection(int m, const double *pos, double *e);
  int BoxInter(double *inter, double *real);     // CalculateEnergy::BoxInter
  int RecipSetup();                              // Ewald::BoxReciprocalSetup
  int RecipSums(const double *d_x, const double *d_y, const double *d_z);
  int RecipEnergy(double *e, bool ref_sums);     // Ewald::BoxReciprocal
  int SystemTotal(double out9[9]);               // CalculateEnergy::SystemTotal
  int MoleculeInter(int m, const double *new_pos, double *lj, double *real,
                    int *overlap);
  int SingleMoleculeInter(int m, const double lam[4], double out[4]);
  int VirialCalc(double out16[16]);              // CalculateEnergy::VirialCalc
  int ParticleInter(int m, int part, const double *trials, int ntrials,
                    double *en, double *real, int *overlap);
  int CellRemoveMol(int m);                      // CellList::RemoveMol
  int CellAddMol(int m);                         // CellList::AddMol
  int MolReciprocal(int m, const double *new_pos, double *de);
  int SwapRecip(int m, const double *pos, bool insert, double *de);
  int UpdateRecip();
  int CopyRecip();
  int BoxSelf(double *e);
  int MolCorrection(int m, double *e);
  int BoxCorrection(double *e);
  int BoxForce(double *inter, double *real, double *h_aF, double *h_mF);
  int BoxForceRecip(double *h_aR, double *h_mR);
  int Torque(double *h_tq);

  // ---- state transfer ----
  int GetCoords(double *xyz, double *com);
  int SetCoords(const double *xyz, const double *com);
  int GetEnergy(double e5[5]);
  int SetEnergy(const double e5[5]);
  int GetCells(int *cell_of_atom, int edge[3]);
  int GetKVectors(double *out7);
  int GetSumNew(double *sr, double *si);
  int CheckError();

  // ---- internals shared with the Monte Carlo loop ----
  DevBox dev{};
  FF ff{};
  FF *d_ff = nullptr;
  BoxConfig cfg;
  HostSystem host;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int sm_count = 0;
  std::string last_error;
  McState *mc = nullptr;
  size_t dev_bytes = 0;  // device memory this box allocated (without mc)
  // molecules taken out of the cell grid by CellRemoveMol (GridAll puts
  // every molecule back); calls that move molecules need all of them in
  std::vector<char> cell_out;
  int n_cell_out = 0;

  // Ewald k-vector sets (dev's k fields mirror kref) and the capacity of the
  // four structure-factor arrays
  KSet kref, knew;
  size_t sums_cap = 0;
  TrialState trial;

  // scratch buffers
  double *d_scratch = nullptr;   // reduction partials
  size_t scratch_len = 0;
  double *h_pinned = nullptr;    // small pinned staging
  double *d_small = nullptr;     // small device staging (positions, results)
  // force buffers: atom/molecule forces, reciprocal forces, torque
  double *d_aF = nullptr, *d_mF = nullptr, *d_aR = nullptr, *d_mR = nullptr,
         *d_tq = nullptr;

  int Fail(int code, const std::string &msg);
  // cell grid of edges L for atoms at host coordinates x, y, z: edges,
  // neighbour table and slot capacity into `d` (arrays grown as needed from
  // `allocs`, capacities in *cell_cap / *nbr_cap)
  int GridGeometry(const double L[3], const double *x, const double *y,
                   const double *z, DevBox &d, size_t *cell_cap,
                   size_t *nbr_cap, std::vector<void *> &allocs);
  int BuildKSet(const double L[3], KSet &ks);
  int EnsureSums(size_t K);
  int TrialCoords(const double L[3], const double *xyz, bool grid);
  int ForceDownload(double *inter, double *real, double *h_aF, double *h_mF);
  bool KSetMatchesEdges() const;
  int new_sums_set_ = 0;  // 1 when the New sums came from the New k set
  void MirrorKRef();
  int CudaCheck(cudaError_t e, const char *what);
  int EnsureScratch(size_t n);
  int Sync();

 private:
  Box() = default;
  int Init(const HostSystem &sys, const BoxConfig &cfg);
  void FreeAll();
  std::vector<void *> allocs_;
  size_t grid_cell_cap_ = 0, grid_nbr_cap_ = 0;
  template <class T>
  int Alloc(T **p, size_t n);
};

// Raise `func`'s dynamic shared-memory limit to at least `bytes`; the limit
// only ever grows, so launches and occupancy queries from several host
// threads never see it lowered under them (gb_box.cu).
void raise_smem_limit(const void *func, size_t bytes);

// host helpers (gb_box.cu)
void build_ff(const HostSystem &s, const BoxConfig &c, FF *ff);
void recip_vectors(const double L[3], double volume, double alphaSq,
                   double recip_rcutSq, double recip_rcut,
                   std::vector<double> &kx, std::vector<double> &ky,
                   std::vector<double> &kz, std::vector<double> &hsqr,
                   std::vector<double> &prefact, std::vector<char4> &kn,
                   int *kmax);

// kernel launchers (gb_cells.cu / gb_real.cu / gb_recip.cu).  Launchers
// that take a DevBox run on that view (coordinates and cell grid), which lets
// the MultiParticle move evaluate its trial state in separate buffers.
int launch_grid_all(Box &b, const DevBox &d);
int launch_box_inter(Box &b, double *d_out2);
int launch_box_inter_view(Box &b, const DevBox &d, double *d_out2);
int launch_box_virial(Box &b, double *d_out6);
int launch_virial_recip(Box &b, double *d_out6);
int launch_recip_sums(Box &b, const double *x, const double *y,
                      const double *z, double *sumR, double *sumI);
int launch_recip_sums_view(Box &b, const DevBox &d, const double *x,
                           const double *y, const double *z, double *sumR,
                           double *sumI);
int launch_recip_sums_ff(Box &b, const double *x, const double *y,
                         const double *z, double *sumR, double *sumI);
int launch_recip_energy(Box &b, const double *sumR, const double *sumI,
                        double *d_out);
int launch_recip_energy_view(Box &b, const DevBox &d, const double *sumR,
                             const double *sumI, double *d_out);
int launch_mol_recip(Box &b, int m, const double *d_newpos, int sign_mode,
                     double *d_out);
int launch_mol_inter(Box &b, int m, const double *d_newpos, double *d_out3);
int launch_single_mol_inter(Box &b, int m, const double *d_lam4,
                            double *d_out4);
int launch_particle_inter(Box &b, int kind, double charge,
                          const double *d_trials, int ntrials, double *d_out);
int launch_cell_remove_mol(Box &b, int m);
int launch_cell_add_mol(Box &b, int m);
int launch_correction(Box &b, double *d_out);
int launch_box_force(Box &b, const DevBox &d, double *aF, double *mF,
                     double *d_out2);
int launch_force_recip(Box &b, const DevBox &d, const double *sumR,
                       const double *sumI, double *aR, double *mR);
int launch_torque(Box &b, const DevBox &d, const double *aF, const double *aR,
                  double *tq);

}  // namespace gb
