// extern "C" entry points (include/gomc_gb300.h) over gb::Box.
#include "gomc_gb300.h"
#include "gb_box.h"
#include "gb_mc.h"

#include <cstring>
#include <string>

struct gb_box {
  gb::Box *b;
};

namespace {
thread_local std::string g_create_error;

int guard_box(gb_box *box) {
  if (!box || !box->b)
    return gb::ERR_ARG;
  return gb::OK;
}

// Every call that works on the box's coordinates needs its k-vector set to
// be the one of its edges; after gb_update_recip_vec swapped in a set for
// other edges, only gb_set_box (with those edges) and the calls below that
// use guard_box are valid.
int guard(gb_box *box) {
  int rc = guard_box(box);
  if (rc)
    return rc;
  if (!box->b->KSetMatchesEdges())
    return box->b->Fail(gb::ERR_STATE,
                        "the k-vector set is for other box edges: call "
                        "gb_set_box with them");
  return gb::OK;
}

// Calls that move molecules or save the cell grid need every molecule in the
// grid (a molecule taken out by gb_cell_remove_mol goes back with
// gb_cell_add_mol or gb_grid_all).
int all_in_grid(gb::Box &b) {
  if (b.n_cell_out)
    return b.Fail(gb::ERR_STATE,
                  "a molecule is out of the cell list (gb_cell_remove_mol)");
  return gb::OK;
}
}  // namespace

namespace gb {
// Message returned by gb_last_error(NULL) for calls that take no box.
void set_api_error(const char *msg) { g_create_error = msg; }
}  // namespace gb

extern "C" {

const char *gb_version(void) { return "gomc_gb300 0.1 (sm_103a)"; }

const char *gb_last_error(const gb_box *box) {
  if (!box || !box->b)
    return g_create_error.c_str();
  return box->b->last_error.c_str();
}

int gb_box_create(const gb_system_desc *sys, const gb_config *cfg,
                  gb_box **out) {
  if (!sys || !cfg || !out || !sys->pos || !sys->atom_kind ||
      !sys->atom_charge || !sys->mol_start || !sys->kind_epsilon ||
      !sys->kind_sigma || !sys->kind_n) {
    g_create_error = "null argument";
    return gb::ERR_ARG;
  }
  if (sys->n_atoms <= 0 || sys->n_mol <= 0 || sys->n_kinds <= 0) {
    g_create_error = "empty system";
    return gb::ERR_ARG;
  }
  gb::HostSystem h;
  h.n_atoms = sys->n_atoms;
  h.n_mol = sys->n_mol;
  h.n_kinds = sys->n_kinds;
  h.x.resize(h.n_atoms);
  h.y.resize(h.n_atoms);
  h.z.resize(h.n_atoms);
  h.q.assign(sys->atom_charge, sys->atom_charge + h.n_atoms);
  h.kind.assign(sys->atom_kind, sys->atom_kind + h.n_atoms);
  h.mstart.assign(sys->mol_start, sys->mol_start + h.n_mol + 1);
  h.eps.assign(sys->kind_epsilon, sys->kind_epsilon + h.n_kinds);
  h.sigma.assign(sys->kind_sigma, sys->kind_sigma + h.n_kinds);
  h.nexp.assign(sys->kind_n, sys->kind_n + h.n_kinds);
  for (int i = 0; i < h.n_atoms; ++i) {
    h.x[i] = sys->pos[3 * i];
    h.y[i] = sys->pos[3 * i + 1];
    h.z[i] = sys->pos[3 * i + 2];
  }
  for (int d = 0; d < 3; ++d)
    h.L[d] = sys->box[d];
  gb::BoxConfig c;
  c.temperature = cfg->temperature;
  c.rcut = cfg->rcut;
  c.rcut_low = cfg->rcut_low;
  c.rcut_coulomb = cfg->rcut_coulomb > 0 ? cfg->rcut_coulomb : cfg->rcut;
  c.tolerance = cfg->tolerance;
  c.ewald = cfg->ewald ? 1 : 0;
  c.electrostatic = cfg->electrostatic ? 1 : 0;
  c.precision = cfg->precision;
  c.device = cfg->device;
  c.sc_alpha = cfg->sc_alpha;
  c.sc_sigma = cfg->sc_sigma;
  c.sc_power = cfg->sc_power;
  c.sc_coul = cfg->sc_coul ? 1 : 0;
  if (c.sc_power < 0) {
    g_create_error = "ScalePower must be >= 0";
    return gb::ERR_ARG;
  }
  if (c.precision != GB_FP64 && c.precision != GB_MIXED) {
    g_create_error = "precision must be GB_FP64 or GB_MIXED";
    return gb::ERR_ARG;
  }
  gb::Box *b = nullptr;
  std::string err;
  int rc = gb::Box::Create(h, c, &b, &err);
  if (rc) {
    g_create_error = err;
    return rc;
  }
  *out = new gb_box{b};
  return gb::OK;
}

void gb_box_destroy(gb_box *box) {
  if (!box)
    return;
  gb::mc_destroy(*box->b);
  delete box->b;
  delete box;
}

#define BOX_CALL(expr)          \
  do {                          \
    int rc_ = guard(box);       \
    if (rc_)                    \
      return rc_;               \
    return box->b->expr;        \
  } while (0)

int gb_system_total(gb_box *box, double *out9) {
  if (!out9)
    return gb::ERR_ARG;
  BOX_CALL(SystemTotal(out9));
}
int gb_box_inter(gb_box *box, double *inter, double *real) {
  if (!inter || !real)
    return gb::ERR_ARG;
  BOX_CALL(BoxInter(inter, real));
}
int gb_molecule_inter(gb_box *box, int32_t mol, const double *new_pos,
                      double *lj, double *real, int32_t *overlap) {
  if (!new_pos || !lj || !real || !overlap)
    return gb::ERR_ARG;
  int ov = 0;
  int rc = guard(box);
  if (rc)
    return rc;
  rc = box->b->MoleculeInter(mol, new_pos, lj, real, &ov);
  *overlap = ov;
  return rc;
}
int gb_mc_autotune(gb_box *box, int32_t objective, int32_t trial_moves,
                   gb_mc_shape *chosen, gb_mc_shape *tried, int32_t cap,
                   int32_t *n_tried) {
  int rc = guard(box);
  if (rc)
    return rc;
  if (cap < 0 || (cap > 0 && !tried))
    return box->b->Fail(gb::ERR_ARG, "tried must hold cap shapes");
  if ((rc = all_in_grid(*box->b)))
    return rc;
  return gb::mc_autotune(*box->b, objective, trial_moves, chosen, tried, cap,
                         n_tried);
}

int gb_checkpoint_size(gb_box *box, int64_t *bytes) {
  int rc = guard(box);
  if (rc)
    return rc;
  if (!bytes)
    return gb::ERR_ARG;
  return gb::checkpoint_size(*box->b, bytes);
}
int gb_checkpoint_save(gb_box *box, void *buf, int64_t bytes) {
  int rc = guard(box);
  if (rc)
    return rc;
  if (!buf)
    return gb::ERR_ARG;
  if ((rc = all_in_grid(*box->b)))
    return rc;
  return gb::checkpoint_save(*box->b, buf, bytes);
}
int gb_checkpoint_load(gb_box *box, const void *buf, int64_t bytes) {
  int rc = guard(box);
  if (rc)
    return rc;
  if (!buf)
    return gb::ERR_ARG;
  if ((rc = all_in_grid(*box->b)))
    return rc;
  return gb::checkpoint_load(*box->b, buf, bytes);
}

int gb_virial(gb_box *box, double *out16) {
  if (!out16)
    return gb::ERR_ARG;
  BOX_CALL(VirialCalc(out16));
}

int gb_single_molecule_inter(gb_box *box, int32_t mol, const double *lambdas4,
                             double *out4) {
  int rc = guard(box);
  if (rc)
    return rc;
  if (!lambdas4 || !out4)
    return box->b->Fail(gb::ERR_ARG, "null lambdas or output");
  return box->b->SingleMoleculeInter(mol, lambdas4, out4);
}

int gb_particle_inter(gb_box *box, int32_t mol, int32_t part,
                      const double *trials, int32_t ntrials, double *en,
                      double *real, int32_t *overlap) {
  if (!trials || !en || !real || !overlap)
    return gb::ERR_ARG;
  int rc = guard(box);
  if (rc)
    return rc;
  std::vector<int> ov(ntrials > 0 ? ntrials : 1, 0);
  rc = box->b->ParticleInter(mol, part, trials, ntrials, en, real, ov.data());
  for (int t = 0; t < ntrials && !rc; ++t)
    overlap[t] = ov[t];
  return rc;
}
int gb_cell_remove_mol(gb_box *box, int32_t mol) { BOX_CALL(CellRemoveMol(mol)); }
int gb_cell_add_mol(gb_box *box, int32_t mol) { BOX_CALL(CellAddMol(mol)); }
int gb_box_force(gb_box *box, double *inter, double *real, double *atom_force,
                 double *mol_force) {
  if (!inter || !real)
    return gb::ERR_ARG;
  BOX_CALL(BoxForce(inter, real, atom_force, mol_force));
}
int gb_calculate_torque(gb_box *box, double *mol_torque) {
  BOX_CALL(Torque(mol_torque));
}
int gb_num_kvectors(gb_box *box, int32_t *k_count, int32_t *kmax) {
  int rc = guard(box);
  if (rc)
    return rc;
  if (k_count)
    *k_count = box->b->cfg.ewald ? box->b->dev.K : 0;
  if (kmax)
    *kmax = box->b->cfg.ewald ? box->b->dev.kmax : 0;
  return gb::OK;
}
int gb_get_kvectors(gb_box *box, double *out7) {
  if (!out7)
    return gb::ERR_ARG;
  BOX_CALL(GetKVectors(out7));
}
int gb_get_sums_new(gb_box *box, double *sum_r, double *sum_i) {
  if (!sum_r || !sum_i)
    return gb::ERR_ARG;
  BOX_CALL(GetSumNew(sum_r, sum_i));
}
int gb_box_reciprocal_setup(gb_box *box) { BOX_CALL(RecipSetup()); }
int gb_box_reciprocal_sums(gb_box *box) {
  BOX_CALL(RecipSums(box->b->dev.x, box->b->dev.y, box->b->dev.z));
}
int gb_box_reciprocal(gb_box *box, int32_t is_new_volume, double *energy) {
  if (!energy)
    return gb::ERR_ARG;
  int rc = guard_box(box);
  if (rc)
    return rc;
  return box->b->RecipEnergyNew(energy, is_new_volume != 0);
}
int gb_box_reciprocal_sums_coords(gb_box *box, const double *xyz) {
  if (!xyz)
    return gb::ERR_ARG;
  BOX_CALL(RecipSumsCoords(xyz, false));
}
int gb_box_reciprocal_setup_coords(gb_box *box, const double *xyz) {
  if (!xyz)
    return gb::ERR_ARG;
  int rc = guard_box(box);
  if (rc)
    return rc;
  return box->b->RecipSumsCoords(xyz, true);
}
int gb_recip_init(gb_box *box, const double *edges3, int32_t *k_count) {
  if (!edges3)
    return gb::ERR_ARG;
  int rc = guard_box(box);
  if (rc || (rc = box->b->RecipInit(edges3)))
    return rc;
  if (k_count)
    *k_count = box->b->cfg.ewald ? box->b->knew.K : 0;
  return gb::OK;
}
int gb_update_recip_vec(gb_box *box) {
  int rc = guard_box(box);
  if (rc)
    return rc;
  return box->b->UpdateRecipVec();
}
int gb_set_box(gb_box *box, const double *edges3, const double *xyz,
               const double *com) {
  if (!edges3 || !xyz)
    return gb::ERR_ARG;
  int rc = guard_box(box);
  if (rc)
    return rc;
  return box->b->SetBox(edges3, xyz, com);
}
int gb_box_edges(gb_box *box, double *edges3) {
  if (!edges3)
    return gb::ERR_ARG;
  int rc = guard_box(box);
  if (rc)
    return rc;
  for (int d = 0; d < 3; ++d)
    edges3[d] = box->b->dev.L[d];
  return gb::OK;
}
int gb_box_inter_coords(gb_box *box, const double *edges3, const double *xyz,
                        double *inter, double *real) {
  if (!edges3 || !xyz || !inter || !real)
    return gb::ERR_ARG;
  int rc = guard_box(box);
  if (rc)
    return rc;
  return box->b->BoxInterAt(edges3, xyz, inter, real);
}
int gb_box_force_coords(gb_box *box, const double *xyz, double *inter,
                        double *real, double *atom_force, double *mol_force) {
  if (!xyz || !inter || !real)
    return gb::ERR_ARG;
  BOX_CALL(BoxForceAt(xyz, inter, real, atom_force, mol_force));
}
int gb_swap_self(gb_box *box, int32_t mol, double *self) {
  if (!self)
    return gb::ERR_ARG;
  BOX_CALL(SwapSelf(mol, self));
}
int gb_swap_correction(gb_box *box, int32_t mol, const double *pos,
                       double *corr) {
  if (!pos || !corr)
    return gb::ERR_ARG;
  BOX_CALL(SwapCorrection(mol, pos, corr));
}
int gb_mol_reciprocal(gb_box *box, int32_t mol, const double *new_pos,
                      double *delta) {
  if (!new_pos || !delta)
    return gb::ERR_ARG;
  BOX_CALL(MolReciprocal(mol, new_pos, delta));
}
int gb_swap_dest_recip(gb_box *box, int32_t mol, const double *pos,
                       double *delta) {
  if (!pos || !delta)
    return gb::ERR_ARG;
  BOX_CALL(SwapRecip(mol, pos, true, delta));
}
int gb_swap_source_recip(gb_box *box, int32_t mol, const double *pos,
                         double *delta) {
  if (!pos || !delta)
    return gb::ERR_ARG;
  BOX_CALL(SwapRecip(mol, pos, false, delta));
}
int gb_update_recip(gb_box *box) { BOX_CALL(UpdateRecip()); }
int gb_copy_recip(gb_box *box) { BOX_CALL(CopyRecip()); }
int gb_box_self(gb_box *box, double *self) {
  if (!self)
    return gb::ERR_ARG;
  BOX_CALL(BoxSelf(self));
}
int gb_mol_correction(gb_box *box, int32_t mol, double *corr) {
  if (!corr)
    return gb::ERR_ARG;
  BOX_CALL(MolCorrection(mol, corr));
}
int gb_box_force_reciprocal(gb_box *box, double *atom_force_rec,
                            double *mol_force_rec) {
  BOX_CALL(BoxForceRecip(atom_force_rec, mol_force_rec));
}
int gb_grid_all(gb_box *box) { BOX_CALL(GridAll()); }
int gb_cell_membership(gb_box *box, int32_t *cell_of_atom, int32_t *edge3) {
  if (!cell_of_atom || !edge3)
    return gb::ERR_ARG;
  BOX_CALL(GetCells(cell_of_atom, edge3));
}
int gb_get_coords(gb_box *box, double *xyz, double *com) {
  BOX_CALL(GetCoords(xyz, com));
}
int gb_set_coords(gb_box *box, const double *xyz, const double *com) {
  if (!xyz)
    return gb::ERR_ARG;
  BOX_CALL(SetCoords(xyz, com));
}
int gb_get_energy(gb_box *box, double *e5) {
  if (!e5)
    return gb::ERR_ARG;
  int rc = guard_box(box);
  if (rc)
    return rc;
  return box->b->GetEnergy(e5);
}
int gb_set_energy(gb_box *box, const double *e5) {
  if (!e5)
    return gb::ERR_ARG;
  int rc = guard_box(box);
  if (rc)
    return rc;
  return box->b->SetEnergy(e5);
}

int gb_mc_init(gb_box *box, const gb_mc_params *p) {
  int rc = guard(box);
  if (rc)
    return rc;
  if (!p)
    return gb::ERR_ARG;
  return gb::mc_init(*box->b, *p);
}
int gb_mc_run(gb_box *box, int64_t first_step, int64_t nsteps, int32_t *kind,
              int32_t *mol, int32_t *accepted, double *de) {
  int rc = guard(box);
  if (rc || (rc = all_in_grid(*box->b)))
    return rc;
  return gb::mc_run(*box->b, first_step, nsteps, kind, mol, accepted, de);
}
int gb_mc_state(gb_box *box, double *scales4, int64_t *counts6) {
  int rc = guard(box);
  if (rc)
    return rc;
  return gb::mc_state(*box->b, scales4, counts6);
}
int gb_mc_timing(gb_box *box, int32_t reset, double *chain_ms,
                 int64_t *chain_launches, int64_t *chain_moves, double *mp_ms,
                 int64_t *mp_moves) {
  int rc = guard(box);
  if (rc)
    return rc;
  return gb::mc_timing(*box->b, reset, chain_ms, chain_launches, chain_moves,
                       mp_ms, mp_moves);
}
int gb_gomc_checkpoint_read(const void *buf, int64_t bytes,
                            gb_gomc_chk *out) {
  return gb::gomc_chk_read(buf, bytes, out);
}
int gb_gomc_checkpoint_write(const void *tmpl, int64_t tmpl_bytes,
                             const gb_gomc_chk *in, void *out,
                             int64_t out_cap, int64_t *out_bytes) {
  return gb::gomc_chk_write(tmpl, tmpl_bytes, in, out, out_cap, out_bytes);
}
int gb_mc_get_gomc_state(gb_box *box, gb_gomc_chk *out) {
  int rc = guard(box);
  if (rc || !out)
    return rc ? rc : gb::ERR_ARG;
  return gb::mc_get_gomc_state(*box->b, out);
}
int gb_mc_set_gomc_state(gb_box *box, const gb_gomc_chk *in) {
  int rc = guard(box);
  if (rc || !in)
    return rc ? rc : gb::ERR_ARG;
  return gb::mc_set_gomc_state(*box->b, in);
}
int gb_mc_set_wait_limit(gb_box *box, int64_t polls) {
  int rc = guard(box);
  if (rc)
    return rc;
  return gb::mc_set_wait_limit(*box->b, polls);
}
int gb_mc_profile(gb_box *box, int32_t enable, double *us13,
                  int64_t *moves2) {
  int rc = guard(box);
  if (rc)
    return rc;
  return gb::mc_profile(*box->b, enable, us13, moves2);
}
int gb_mc_drift(gb_box *box, double *max4, double *last4, int64_t *n) {
  int rc = guard(box);
  if (rc)
    return rc;
  if (!box->b->mc)
    return gb::ERR_STATE;
  gb::McState &s = *box->b->mc;
  for (int i = 0; i < 4; ++i) {
    if (max4)
      max4[i] = s.drift_max[i];
    if (last4)
      last4[i] = s.drift_last[i];
  }
  if (n)
    *n = s.recomputes;
  return gb::OK;
}
int gb_mc_layout(gb_box *box, int32_t *ctas_per_chain,
                 int32_t *max_concurrent, int64_t *smem_bytes) {
  int rc = guard(box);
  if (rc)
    return rc;
  gb::Box &b = *box->b;
  if (!b.mc)
    return b.Fail(gb::ERR_STATE, "gb_mc_init has not been called");
  gb::McState &s = *b.mc;
  int per = 1, conc = 1;
  size_t sm = 0;
  if (b.cfg.precision == GB_MIXED) {
    per = s.cluster;
    sm = s.mixed_smem;
    conc = gb::max_active_clusters(s.cluster, s.mixed_smem);
  } else {
    per = s.grid;
  }
  if (ctas_per_chain)
    *ctas_per_chain = per;
  if (max_concurrent)
    *max_concurrent = conc;
  if (smem_bytes)
    *smem_bytes = (int64_t)sm;
  return gb::OK;
}
int gb_mc_shape_get(gb_box *box, gb_mc_shape *shape) {
  int rc = guard(box);
  if (rc)
    return rc;
  gb::Box &b = *box->b;
  if (!shape)
    return b.Fail(gb::ERR_ARG, "shape is NULL");
  if (!b.mc)
    return b.Fail(gb::ERR_STATE, "gb_mc_init has not been called");
  gb::McState &s = *b.mc;
  *shape = gb_mc_shape{};
  if (b.cfg.precision == GB_MIXED) {
    shape->ctas = s.cluster;
    shape->unit_lanes = 1 << s.ulog;
    shape->max_concurrent = gb::max_active_clusters(s.cluster, s.mixed_smem);
  } else {
    shape->ctas = s.grid;
    shape->writer_kchunk = s.params.writer_kchunk;
    shape->moves_in_flight = s.pipe ? 2 : 1;
    shape->max_concurrent = 1;
  }
  return gb::OK;
}
int gb_box_stream(gb_box *box, void **stream) {
  int rc = guard(box);
  if (rc)
    return rc;
  if (!stream)
    return gb::ERR_ARG;
  *stream = (void *)box->b->stream;
  return gb::OK;
}
int gb_mc_run_batch(gb_box **boxes, int32_t nboxes, int64_t first_step,
                    int64_t nsteps) {
  if (!boxes || nboxes <= 0)
    return gb::ERR_ARG;
  std::vector<gb::Box *> v;
  for (int i = 0; i < nboxes; ++i) {
    if (!boxes[i] || !boxes[i]->b)
      return gb::ERR_ARG;
    int rc = all_in_grid(*boxes[i]->b);
    if (rc)
      return rc;
    v.push_back(boxes[i]->b);
  }
  return gb::mc_run_batch(v, first_step, nsteps);
}

}  // extern "C"
