// Continuous-batching job server: many independent mixed-precision NVT
// simulations on one GPU, each resident in HBM from admission to completion.
//
// A round (Server::Round) does, in order:
//   1. launch: every resident job runs its next segment (at most its
//      quantum of moves, cut at its next FP64 recompute boundary).  Jobs are grouped by
//      cluster size; each group is one kernel launch, the groups run on
//      separate streams and overlap on the device (mixed_launch);
//   2. admission, while those kernels run: queued jobs, first come first
//      served, are admitted if their estimated device memory fits the budget
//      and their chains fit the free CTA slots;
//   3. completion: wait for the launches and record sweep completions.
// Building an admitted job's box (coordinates, cell grid, k-vectors,
// structure factors, initial FP64 energies) and the periodic FP64
// recomputes that fall due run on helper threads, on the jobs' own
// streams, beside the rounds; a job sits out rounds meanwhile.  Finished
// jobs are retired at the start of the next round (final coordinates and
// energies copied to the host, device memory returned to the budget).
// A job's segment lengths depend only on the job (its quantum, recompute
// frequency and step count), and its cluster size only on its own size, so
// it computes the same moves with the same arithmetic alone or in any mix.
//
// This has no counterpart in the reference, which runs one simulation per
// process (src/Simulation.cpp:116-168).
#include "gomc_gb300.h"
#include "gb_box.h"
#include "gb_mc.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace gb {

namespace {

using Clock = std::chrono::steady_clock;

struct Job {
  int64_t id = 0;
  HostSystem host;
  BoxConfig cfg;
  gb_mc_params mc{};
  int64_t nsteps = 0, sweep = 0, done = 0;
  int status = GB_JOB_QUEUED;
  int csize = 0;
  int64_t quantum = 0;  // moves per round
  size_t smem = 0;      // dynamic shared memory per CTA
  size_t mem = 0;   // admission estimate, or the box's bytes when larger
  bool busy = false;  // being set up or recomputed: sits out rounds
  int K = -1, kmax = 0;  // k-vectors and largest |n|, once known
  Box *box = nullptr;
  double t_submit = 0, t_admit = 0, t_done = 0, t_last = 0;
  std::vector<double> xyz, com;
  double e5[5] = {0, 0, 0, 0, 0};
  std::string msg;
};

// CTA-slot model of one GPU for admission: an SM holds as many chain CTAs as
// its shared memory and registers allow.
struct Slots {
  int sms = 0;
  size_t smem_per_sm = 0;
};

}  // namespace

struct Server {
  gb_server_config cfg{};
  Slots slots;
  size_t budget = 0, mem_used = 0;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<Job *> queue;     // submitted, not yet admitted
  std::vector<Job *> resident; // admitted (being set up, running, recomputing)
  std::deque<Job *> tasks;     // set-up and recompute work for the helper
  std::map<int64_t, Job *> jobs;
  int64_t next_id = 1;
  Clock::time_point t0;
  std::thread worker;
  std::vector<std::thread> helpers;  // set-up / recompute threads
  bool worker_on = false, stop = false, abort = false;
  int worker_rc = OK;
  std::string last_error;
  // statistics
  std::vector<double> sweep_lat;  // seconds
  int64_t moves = 0, rounds = 0, resident_sum = 0;
  // occupancy sums over rounds, taken after each round's admission: jobs
  // admitted, CTA-slot and shared-memory fractions in use, jobs queued
  double occ_admitted = 0, occ_ctas = 0, occ_smem = 0, occ_queued = 0;
  int64_t occ_rounds = 0;
  // admissions stopped at the queue's head by device memory, by shared
  // memory, by CTA count
  int64_t stop_mem = 0, stop_smem = 0, stop_ctas = 0;
  // launch balance: per round, the chain CTAs' kernel time over the time
  // they were held (the longest launch of the round), CTA-weighted; and the
  // round's wall time outside its longest launch (host work, launch gaps)
  double bal_sum = 0, gap_s = 0;
  double t_first = -1, t_last_done = 0;
  double helper_s = 0, round_s = 0;  // time in set-up / recompute, in rounds

  double Now() const {
    return std::chrono::duration<double>(Clock::now() - t0).count();
  }
  int Fail(int code, const std::string &m) {
    std::lock_guard<std::mutex> g(mu);
    last_error = m;
    return code;
  }
  int Round(int32_t *pending, bool *worked);
  int Admit();
  void SlotUse(size_t *smem, int *ctas) const;
  void RunTask(Job *j);
  void RunTasksInline();
  void Retire(Job *j);
  void Worker();
  void Helper();
};

namespace {

// Cluster size of a job: the smallest cluster whose CTAs hold at most 2048
// k-vectors each (a job's choice depends on its own size only), at least 2.
int job_cluster(const Job &j, int K) {
  if (j.mc.cluster_size > 0)
    return j.mc.cluster_size;
  for (int c : {2, 4, 8, 16})
    if ((K + c - 1) / c <= 2048)
      return c;
  return 16;
}

// Moves per round of a job: `quantum` scaled by the time of a move of a
// chain with 4,096 k-vectors per CTA over the time of one of this job's, so
// that every resident job's segment takes about the same time and no chain
// idles while the round waits for the slowest.  A move costs a fixed part
// (the cluster barriers, the header, the real-space pairs: about as long as
// 2,560 k-vectors of one CTA's reciprocal work on GB300) plus its k-vectors
// per CTA.  Within [quantum / 4, 8 quantum]; depends on the job alone.
int64_t job_quantum(int quantum, int K, int csize) {
  constexpr int64_t FIXED = 2560, REF = 4096;
  int64_t per_cta = std::max(K / std::max(csize, 1), 256);
  int64_t q = (int64_t)quantum * (FIXED + REF) / (FIXED + per_cta);
  return std::min<int64_t>(std::max<int64_t>(q, std::max(quantum / 4, 1)),
                           8 * (int64_t)quantum);
}

// k-vector count and largest |n| of a box, from the set-up rules of
// Box::Init (recip_vectors on the host; no device work).
void job_kvectors(const Job &j, int *K, int *kmax) {
  FF ff;
  build_ff(j.host, j.cfg, &ff);
  std::vector<double> kx, ky, kz, hs, pf;
  std::vector<char4> kn;
  double vol = j.host.L[0] * j.host.L[1] * j.host.L[2];
  *K = 0;
  *kmax = 0;
  if (!j.cfg.ewald)
    return;
  recip_vectors(j.host.L, vol, ff.alphaSq, ff.recip_rcutSq, ff.recip_rcut, kx,
                ky, kz, hs, pf, kn, kmax);
  *K = (int)kx.size();
}

// Device bytes the job's box will hold (Box::Init + mc_init in the mixed
// form, the move buffer sized to `moves`), from the same sizing rules.
size_t job_bytes(const Job &j, int K, int kmax, int csize, size_t moves) {
  const HostSystem &s = j.host;
  size_t N = s.n_atoms, M = s.n_mol;
  int edge[3];
  size_t ncell = 1;
  for (int d = 0; d < 3; ++d) {
    edge[d] = std::max((int)std::floor(s.L[d] / j.cfg.rcut), 3);
    ncell *= edge[d];
  }
  // slot capacity: three times the fullest cell, as Box::Init
  std::vector<int> cnt(ncell, 0);
  int mx = 0;
  for (size_t i = 0; i < N; ++i) {
    double p[3] = {wrap1(s.x[i], s.L[0]), wrap1(s.y[i], s.L[1]),
                   wrap1(s.z[i], s.L[2])};
    int c[3];
    for (int d = 0; d < 3; ++d) {
      c[d] = (int)(p[d] / (s.L[d] / edge[d]));
      c[d] -= c[d] == edge[d] ? 1 : 0;
    }
    mx = std::max(mx, ++cnt[((size_t)c[0] * edge[1] + c[1]) * edge[2] + c[2]]);
  }
  size_t cap = (std::max(3 * mx, 32) + 31) / 32 * 32;
  size_t NC = ncell * cap;
  size_t slot = 4 + 32 + 4 + 16 + 4;  // atom, pos, meta, fix, qlo
  size_t box = N * (3 * 8 + 8 + 4 * 4 + 6 * 8) + M * (3 * 8 + 4 + 9 * 8) +
               ncell * (4 + NB27 * 4) + NC * slot + (size_t)K * (9 * 8 + 8) +
               2 * 12 * 64 * (ETAB_DEG + 1) * 8 +  // erfc and force tables
               sizeof(FF) + 256;
  size_t mc = moves * (sizeof(MoveRec) + 12 * 8) +
              N * (3 * 8 + 6 * 8 + 8) + M * (3 * 8 + 12 * 8 + 4) +
              NC * slot + ncell * 4 + 256 * sizeof(MixedChain) +
              (size_t)(2 * MAX_MOL_ATOMS * 3) * (kmax + 1) * 16 + 64 * 1024;
  if (mixed_smem(K, kmax, csize, true) > MIXED_SMEM_MAX)
    mc += mixed_cold_buffer(K, csize);
  // reduction scratch of the set-up kernels and allocation rounding
  size_t scratch = (size_t)K * 16 + N * 8 + ((size_t)1 << 20);
  return box + mc + scratch + 96 * 512;
}

// A job's host-side system and configuration, copied from the C structures.
Job *make_job(const gb_system_desc *sys, const gb_config *cfg) {
  auto *j = new Job();
  HostSystem &h = j->host;
  h.n_atoms = sys->n_atoms;
  h.n_mol = sys->n_mol;
  h.n_kinds = sys->n_kinds;
  h.x.resize(h.n_atoms);
  h.y.resize(h.n_atoms);
  h.z.resize(h.n_atoms);
  for (int i = 0; i < h.n_atoms; ++i) {
    h.x[i] = sys->pos[3 * i];
    h.y[i] = sys->pos[3 * i + 1];
    h.z[i] = sys->pos[3 * i + 2];
  }
  h.q.assign(sys->atom_charge, sys->atom_charge + h.n_atoms);
  h.kind.assign(sys->atom_kind, sys->atom_kind + h.n_atoms);
  h.mstart.assign(sys->mol_start, sys->mol_start + h.n_mol + 1);
  h.eps.assign(sys->kind_epsilon, sys->kind_epsilon + h.n_kinds);
  h.sigma.assign(sys->kind_sigma, sys->kind_sigma + h.n_kinds);
  h.nexp.assign(sys->kind_n, sys->kind_n + h.n_kinds);
  for (int d = 0; d < 3; ++d)
    h.L[d] = sys->box[d];
  BoxConfig &c = j->cfg;
  c.temperature = cfg->temperature;
  c.rcut = cfg->rcut;
  c.rcut_low = cfg->rcut_low;
  c.rcut_coulomb = cfg->rcut_coulomb > 0 ? cfg->rcut_coulomb : cfg->rcut;
  c.tolerance = cfg->tolerance;
  c.ewald = cfg->ewald ? 1 : 0;
  c.electrostatic = cfg->electrostatic ? 1 : 0;
  c.precision = GB_MIXED;
  c.device = cfg->device;
  c.sc_alpha = cfg->sc_alpha;
  c.sc_sigma = cfg->sc_sigma;
  c.sc_power = cfg->sc_power;
  c.sc_coul = cfg->sc_coul ? 1 : 0;
  return j;
}

// Admission estimate of a job: k-vectors, cluster size, device bytes.
size_t job_estimate(const Job &j, int quantum, int *csize_out) {
  int K, kmax;
  job_kvectors(j, &K, &kmax);
  int csize = job_cluster(j, K);
  if (csize_out)
    *csize_out = csize;
  return job_bytes(j, K, kmax, csize,
                   (size_t)job_quantum(quantum, K, csize));
}

}  // namespace

// Shared memory (with the runtime's 1 KB per CTA) and CTAs held by the
// resident jobs' chains; the caller holds `mu`.
void Server::SlotUse(size_t *smem, int *ctas) const {
  *smem = 0;
  *ctas = 0;
  for (const Job *r : resident) {
    *smem += (size_t)r->csize * (r->smem + 1024);
    *ctas += r->csize;
  }
}

// Admission (first come first served): reserve the job's estimated device
// memory and CTA slots, mark it resident and busy, and queue its set-up for
// the helpers.  Returns how many jobs were admitted.
int Server::Admit() {
  int admitted = 0;
  for (;;) {
    Job *j = nullptr;
    {
      std::lock_guard<std::mutex> g(mu);
      if (queue.empty())
        break;
      j = queue.front();
    }
    if (j->K < 0)  // host work, done once per job
      job_kvectors(*j, &j->K, &j->kmax);
    const int K = j->K, kmax = j->kmax;
    int csize = job_cluster(*j, K);
    bool cold_smem = mixed_smem(K, kmax, csize, true) <= MIXED_SMEM_MAX;
    size_t smem = mixed_smem(K, kmax, csize, cold_smem);
    size_t est =
      job_bytes(*j, K, kmax, csize, (size_t)job_quantum(cfg.quantum, K, csize));
    std::lock_guard<std::mutex> g(mu);
    // CTA slots: shared memory and two CTAs per SM by registers
    size_t used_smem = 0;
    int used_ctas = 0;
    SlotUse(&used_smem, &used_ctas);
    bool fits_mem = mem_used + est <= budget;
    bool fits_smem = used_smem + (size_t)csize * (smem + 1024) <=
                     slots.smem_per_sm * slots.sms;
    bool fits_ctas = used_ctas + csize <= 2 * slots.sms;
    bool fits_slots = fits_smem && fits_ctas;
    bool fits_count =
        cfg.max_resident <= 0 || (int)resident.size() < cfg.max_resident;
    if (!(fits_mem && fits_slots && fits_count)) {
      if (resident.empty() && est > budget) {
        // can never fit: fail it rather than block the queue
        queue.pop_front();
        j->status = GB_JOB_FAILED;
        j->msg = "job needs more device memory than the server's budget";
        continue;
      }
      stop_mem += fits_mem ? 0 : 1;
      stop_smem += fits_smem ? 0 : 1;
      stop_ctas += fits_ctas ? 0 : 1;
      break;
    }
    queue.pop_front();
    j->csize = csize;
    j->quantum = job_quantum(cfg.quantum, K, csize);
    j->smem = smem;
    j->mem = est;
    j->busy = true;
    mem_used += est;
    resident.push_back(j);
    tasks.push_back(j);
    admitted++;
  }
  if (admitted)
    cv.notify_all();
  return admitted;
}

// Set-up of an admitted job (its box: coordinates, cell grid, k-vectors,
// structure factors and the initial FP64 energies) or its periodic FP64
// recompute; runs on a helper thread beside the rounds.
void Server::RunTask(Job *j) {
  int rc;
  std::string err;
  double t0 = Now();
  if (!j->box) {
    Box *b = nullptr;
    gb_mc_params p = j->mc;
    p.cluster_size = j->csize;
    p.move_buffer = (int32_t)j->quantum;
    rc = Box::Create(j->host, j->cfg, &b, &err);
    if (!rc && (rc = mc_init(*b, p)))
      err = b->last_error;
    std::lock_guard<std::mutex> g(mu);
    if (rc) {
      if (b) {
        mc_destroy(*b);
        delete b;
      }
      j->status = GB_JOB_FAILED;
      j->msg = err;
      mem_used -= j->mem;
      resident.erase(std::find(resident.begin(), resident.end(), j));
    } else {
      j->box = b;
      size_t actual = b->dev_bytes + b->mc->bytes;
      if (actual > j->mem) {
        mem_used += actual - j->mem;
        j->mem = actual;
      }
      j->smem = b->mc->mixed_smem;
      j->status = GB_JOB_RUNNING;
      j->t_admit = j->t_last = Now();
      if (t_first < 0)
        t_first = j->t_admit;
      j->busy = false;
    }
    helper_s += Now() - t0;
    cv.notify_all();
    return;
  } else {
    rc = mc_recompute(*j->box);
    if (rc)
      err = j->box->last_error;
    std::lock_guard<std::mutex> g(mu);
    if (rc) {
      j->status = GB_JOB_FAILED;
      j->msg = err;
      j->done = j->nsteps;  // retired by the next round
    }
    j->busy = false;
  }
  helper_s += Now() - t0;
  cv.notify_all();
}

void Server::RunTasksInline() {
  for (;;) {
    Job *j = nullptr;
    {
      std::lock_guard<std::mutex> g(mu);
      if (tasks.empty())
        return;
      j = tasks.front();
      tasks.pop_front();
    }
    RunTask(j);
  }
}

// A finished job: final coordinates and running energies to the host, device
// memory back to the budget.
void Server::Retire(Job *j) {
  j->xyz.resize(3 * (size_t)j->host.n_atoms);
  j->com.resize(3 * (size_t)j->host.n_mol);
  int rc = OK;
  if (j->status != GB_JOB_FAILED) {
    rc = j->box->GetCoords(j->xyz.data(), j->com.data());
    if (!rc)
      rc = j->box->GetEnergy(j->e5);
  }
  std::string err = rc ? j->box->last_error : std::string();
  mc_destroy(*j->box);
  delete j->box;
  std::lock_guard<std::mutex> g(mu);
  j->box = nullptr;
  mem_used -= j->mem;
  j->t_done = Now();
  t_last_done = j->t_done;
  if (j->status != GB_JOB_FAILED) {
    j->status = rc ? GB_JOB_FAILED : GB_JOB_DONE;
    j->msg = err;
  }
  resident.erase(std::find(resident.begin(), resident.end(), j));
  cv.notify_all();
}

// One scheduling round (see the top of this file).  *pending = jobs queued or
// resident afterwards; *worked = whether anything was launched or admitted.
int Server::Round(int32_t *pending, bool *worked) {
  int rc;
  bool inline_tasks;
  std::vector<Job *> live, finished;
  {
    std::lock_guard<std::mutex> g(mu);
    inline_tasks = helpers.empty();
    for (Job *j : resident)
      if (!j->busy)
        (j->done >= j->nsteps ? finished : live).push_back(j);
  }
  for (Job *j : finished)
    Retire(j);
  // 1. launch the segments of the jobs that are ready
  std::vector<Box *> boxes;
  std::vector<int64_t> n;
  for (Job *j : live) {
    boxes.push_back(j->box);
    n.push_back(mixed_segment_limit(
        *j->box, std::min<int64_t>(j->quantum, j->nsteps - j->done)));
  }
  std::vector<Box *> leaders;
  double t_start = Now();
  if (!boxes.empty() && (rc = mixed_launch(boxes, n, &leaders)))
    return Fail(rc, "launch: " + boxes[0]->last_error);
  // 2. admission while they run
  int admitted = Admit();
  {
    std::lock_guard<std::mutex> g(mu);
    size_t used_smem;
    int used_ctas;
    SlotUse(&used_smem, &used_ctas);
    occ_admitted += (double)resident.size();
    occ_ctas += (double)used_ctas / (double)(2 * slots.sms);
    occ_smem += (double)used_smem / (double)(slots.smem_per_sm * slots.sms);
    occ_queued += (double)queue.size();
    occ_rounds++;
  }
  if (inline_tasks)
    RunTasksInline();
  // 3. completion; due recomputes go to the helpers
  if (!boxes.empty()) {
    std::vector<char> due;
    if ((rc = mixed_complete(boxes, n, leaders, &due)))
      return Fail(rc, "round: " + boxes[0]->last_error);
    double t_end = Now();
    // each leader's launch time this round (and its events released)
    double ms_max = 0, cta_ms = 0;
    int64_t ctas = 0;
    for (Box *L : leaders) {
      double ms = 0;
      if ((rc = mc_timing(*L, 1, &ms, nullptr, nullptr, nullptr, nullptr)))
        return Fail(rc, "round: " + L->last_error);
      int c = L->mc->cluster, nb = 0;
      for (Box *b : boxes)
        nb += b->mc->cluster == c ? 1 : 0;
      ms_max = std::max(ms_max, ms);
      cta_ms += ms * c * nb;
      ctas += (int64_t)c * nb;
    }
    std::lock_guard<std::mutex> g(mu);
    if (ms_max > 0 && ctas > 0) {
      bal_sum += cta_ms / (ms_max * (double)ctas);
      gap_s += std::max(0.0, t_end - t_start - 1e-3 * ms_max);
    }
    round_s += t_end - t_start;
    rounds++;
    resident_sum += (int64_t)live.size();
    for (size_t i = 0; i < live.size(); ++i) {
      Job *j = live[i];
      int64_t before = j->done, after = before + n[i];
      // sweep completions, placed within the round by move count
      for (int64_t k = before / j->sweep + 1; k * j->sweep <= after; ++k) {
        double t = t_start + (double)(k * j->sweep - before) / (double)n[i] *
                                 (t_end - t_start);
        sweep_lat.push_back(t - j->t_last);
        j->t_last = t;
      }
      j->done = after;
      moves += n[i];
      if (due[i]) {
        j->busy = true;
        tasks.push_back(j);
      }
    }
    cv.notify_all();
  }
  if (inline_tasks)
    RunTasksInline();
  std::lock_guard<std::mutex> g(mu);
  if (pending)
    *pending = (int32_t)(queue.size() + resident.size());
  if (worked)
    *worked = !boxes.empty() || admitted > 0 || !finished.empty();
  cv.notify_all();
  return OK;
}

void Server::Worker() {
  cudaSetDevice(cfg.device);
  for (;;) {
    {
      std::unique_lock<std::mutex> lk(mu);
      if (abort || (stop && queue.empty() && resident.empty()))
        return;
    }
    int32_t pending = 0;
    bool worked = false;
    int rc = Round(&pending, &worked);
    std::unique_lock<std::mutex> lk(mu);
    if (rc) {
      worker_rc = rc;
      abort = true;
      cv.notify_all();
      return;
    }
    if (!worked)  // everything resident is being set up or recomputed
      cv.wait_for(lk, std::chrono::milliseconds(2));
  }
}

void Server::Helper() {
  cudaSetDevice(cfg.device);
  for (;;) {
    Job *j = nullptr;
    {
      std::unique_lock<std::mutex> lk(mu);
      cv.wait(lk, [&] { return abort || !tasks.empty() || !worker_on; });
      if (abort || (tasks.empty() && !worker_on))
        return;
      j = tasks.front();
      tasks.pop_front();
    }
    RunTask(j);
  }
}

}  // namespace gb

struct gb_server {
  gb::Server s;
};

namespace {
gb::Job *find_job(gb_server *srv, int64_t id) {
  auto it = srv->s.jobs.find(id);
  return it == srv->s.jobs.end() ? nullptr : it->second;
}

// Inputs a server job must have (the same checks gb_box_create makes, plus
// the server's own limits).
int check_job(gb_server *srv, const gb_system_desc *sys, const gb_config *cfg,
              const gb_mc_params *mc) {
  if (!srv || !sys || !cfg || !mc || !sys->pos || !sys->atom_kind ||
      !sys->atom_charge || !sys->mol_start || !sys->kind_epsilon ||
      !sys->kind_sigma || !sys->kind_n)
    return gb::ERR_ARG;
  gb::Server &s = srv->s;
  if (sys->n_atoms <= 0 || sys->n_mol <= 0 || sys->n_kinds <= 0 ||
      sys->n_kinds > gb::MAX_KINDS)
    return s.Fail(gb::ERR_ARG, "empty job or kind count out of range");
  if (cfg->precision != GB_MIXED)
    return s.Fail(gb::ERR_UNSUPPORTED, "the server runs mixed-precision jobs");
  if (mc->frac[2] > 0)
    return s.Fail(gb::ERR_UNSUPPORTED,
                  "the server runs translate / rotate moves only");
  if (cfg->device != s.cfg.device)
    return s.Fail(gb::ERR_ARG, "job device differs from the server's");
  return gb::OK;
}
}  // namespace

extern "C" {

int gb_server_create(const gb_server_config *cfg, gb_server **out) {
  if (!cfg || !out)
    return gb::ERR_ARG;
  auto *srv = new gb_server();
  gb::Server &s = srv->s;
  s.cfg = *cfg;
  if (s.cfg.quantum <= 0)
    s.cfg.quantum = 1000;
  if (cudaSetDevice(s.cfg.device) != cudaSuccess) {
    delete srv;
    return gb::ERR_CUDA;
  }
  cudaDeviceProp prop;
  size_t free_b = 0, total_b = 0;
  if (cudaGetDeviceProperties(&prop, s.cfg.device) != cudaSuccess ||
      cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
    delete srv;
    return gb::ERR_CUDA;
  }
  s.slots.sms = prop.multiProcessorCount;
  s.slots.smem_per_sm = prop.sharedMemPerMultiprocessor;
  s.budget = cfg->mem_budget > 0 ? (size_t)cfg->mem_budget
                                 : (size_t)(0.9 * (double)free_b);
  s.t0 = gb::Clock::now();
  *out = srv;
  return gb::OK;
}

void gb_server_destroy(gb_server *srv) {
  if (!srv)
    return;
  gb::Server &s = srv->s;
  {
    std::lock_guard<std::mutex> g(s.mu);
    s.stop = true;
    s.queue.clear();
  }
  s.cv.notify_all();
  // a running round or task finishes; resident jobs are dropped after it
  {
    std::lock_guard<std::mutex> g(s.mu);
    s.abort = true;
  }
  s.cv.notify_all();
  if (s.worker.joinable())
    s.worker.join();
  for (auto &h : s.helpers)
    h.join();
  s.helpers.clear();
  for (auto &kv : s.jobs) {
    gb::Job *j = kv.second;
    if (j->box) {
      gb::mc_destroy(*j->box);
      delete j->box;
    }
    delete j;
  }
  delete srv;
}

int gb_server_submit(gb_server *srv, const gb_system_desc *sys,
                     const gb_config *cfg, const gb_mc_params *mc,
                     int64_t nsteps, int64_t sweep_moves, int64_t *job_id) {
  if (!srv || !job_id)
    return gb::ERR_ARG;
  gb::Server &s = srv->s;
  if (nsteps <= 0)
    return s.Fail(gb::ERR_ARG, "a job needs at least one move");
  int rc = check_job(srv, sys, cfg, mc);
  if (rc)
    return rc;
  auto *j = gb::make_job(sys, cfg);
  j->mc = *mc;
  j->nsteps = nsteps;
  j->sweep = sweep_moves > 0 ? sweep_moves : j->host.n_mol;
  std::lock_guard<std::mutex> g(s.mu);
  j->id = s.next_id++;
  j->t_submit = s.Now();
  s.jobs[j->id] = j;
  s.queue.push_back(j);
  *job_id = j->id;
  s.cv.notify_all();
  return gb::OK;
}

int gb_server_estimate(gb_server *srv, const gb_system_desc *sys,
                       const gb_config *cfg, const gb_mc_params *mc,
                       int64_t *bytes, int32_t *ctas_per_chain) {
  if (!srv || !bytes)
    return gb::ERR_ARG;
  int rc = check_job(srv, sys, cfg, mc);
  if (rc)
    return rc;
  gb::Job *j = gb::make_job(sys, cfg);
  j->mc = *mc;
  int csize = 0;
  *bytes = (int64_t)gb::job_estimate(*j, srv->s.cfg.quantum, &csize);
  if (ctas_per_chain)
    *ctas_per_chain = csize;
  delete j;
  return gb::OK;
}

int gb_server_step(gb_server *srv, int32_t *pending) {
  if (!srv)
    return gb::ERR_ARG;
  gb::Server &s = srv->s;
  {
    std::lock_guard<std::mutex> g(s.mu);
    if (s.worker_on)
      return gb::ERR_STATE;
  }
  cudaSetDevice(s.cfg.device);
  return s.Round(pending, nullptr);
}

int gb_server_start(gb_server *srv) {
  if (!srv)
    return gb::ERR_ARG;
  gb::Server &s = srv->s;
  std::lock_guard<std::mutex> g(s.mu);
  if (s.worker_on)
    return gb::ERR_STATE;
  s.worker_on = true;
  s.stop = false;
  s.worker = std::thread([&s] { s.Worker(); });
  // two helpers: a small job's set-up leaves most of the GPU idle, so two
  // overlap; more only contend for the FP64 units
  for (int i = 0; i < 2; ++i)
    s.helpers.emplace_back([&s] { s.Helper(); });
  return gb::OK;
}

int gb_server_drain(gb_server *srv, double timeout_s) {
  if (!srv)
    return gb::ERR_ARG;
  gb::Server &s = srv->s;
  {
    std::unique_lock<std::mutex> lk(s.mu);
    if (!s.worker_on)
      return gb::ERR_STATE;
    auto done = [&] {
      return (s.queue.empty() && s.resident.empty()) || s.abort;
    };
    if (timeout_s > 0) {
      if (!s.cv.wait_for(lk, std::chrono::duration<double>(timeout_s), done))
        return gb::ERR_TIMEOUT;
    } else {
      s.cv.wait(lk, done);
    }
    s.stop = true;
  }
  s.cv.notify_all();
  s.worker.join();
  {
    std::lock_guard<std::mutex> g(s.mu);
    s.worker_on = false;  // the helpers return once the queue is empty
  }
  s.cv.notify_all();
  for (auto &h : s.helpers)
    h.join();
  s.helpers.clear();
  std::lock_guard<std::mutex> g(s.mu);
  return s.worker_rc;
}

int gb_server_job(gb_server *srv, int64_t job, int32_t *status,
                  int64_t *steps_done, double *times3) {
  if (!srv)
    return gb::ERR_ARG;
  std::lock_guard<std::mutex> g(srv->s.mu);
  gb::Job *j = find_job(srv, job);
  if (!j)
    return gb::ERR_ARG;
  if (status)
    *status = j->status;
  if (steps_done)
    *steps_done = j->done;
  if (times3) {
    times3[0] = j->t_submit;
    times3[1] = j->t_admit;
    times3[2] = j->t_done;
  }
  return gb::OK;
}

int gb_server_result(gb_server *srv, int64_t job, double *xyz, double *com,
                     double *energy5) {
  if (!srv)
    return gb::ERR_ARG;
  std::lock_guard<std::mutex> g(srv->s.mu);
  gb::Job *j = find_job(srv, job);
  if (!j)
    return gb::ERR_ARG;
  if (j->status == GB_JOB_FAILED) {
    srv->s.last_error = j->msg;
    return gb::ERR_STATE;
  }
  if (j->status != GB_JOB_DONE)
    return gb::ERR_STATE;
  if (xyz)
    std::copy(j->xyz.begin(), j->xyz.end(), xyz);
  if (com)
    std::copy(j->com.begin(), j->com.end(), com);
  if (energy5)
    std::copy(j->e5, j->e5 + 5, energy5);
  return gb::OK;
}

int gb_server_stats(gb_server *srv, double *out12) {
  if (!srv || !out12)
    return gb::ERR_ARG;
  double *out10 = out12;
  gb::Server &s = srv->s;
  std::lock_guard<std::mutex> g(s.mu);
  std::vector<double> lat = s.sweep_lat, jl;
  int64_t ndone = 0;
  for (auto &kv : s.jobs)
    if (kv.second->status == GB_JOB_DONE) {
      ndone++;
      jl.push_back(kv.second->t_done - kv.second->t_submit);
    }
  auto pct = [](std::vector<double> &v, double p) {
    if (v.empty())
      return 0.0;
    std::sort(v.begin(), v.end());
    size_t i = (size_t)std::ceil(p * (double)v.size()) - 1;
    return v[std::min(i, v.size() - 1)];
  };
  double wall = s.t_first >= 0 ? s.t_last_done - s.t_first : 0.0;
  out10[0] = (double)ndone;
  out10[1] = (double)s.moves;
  out10[2] = wall;
  out10[3] = wall > 0 ? (double)s.moves / wall : 0.0;
  out10[4] = pct(lat, 0.50) * 1e3;
  out10[5] = pct(lat, 0.99) * 1e3;
  out10[6] = pct(jl, 0.50);
  out10[7] = pct(jl, 0.99);
  out10[8] = (double)s.rounds;
  out10[9] = s.rounds ? (double)s.resident_sum / (double)s.rounds : 0.0;
  out12[10] = s.helper_s;
  out12[11] = s.round_s;
  return gb::OK;
}

int gb_server_occupancy(gb_server *srv, double *out10) {
  if (!srv || !out10)
    return gb::ERR_ARG;
  gb::Server &s = srv->s;
  std::lock_guard<std::mutex> g(s.mu);
  double n = s.occ_rounds ? (double)s.occ_rounds : 1.0;
  double *out5 = out10, *out8 = out10;
  out5[0] = s.occ_admitted / n;
  out5[1] = s.rounds ? (double)s.resident_sum / (double)s.rounds : 0.0;
  out5[2] = s.occ_ctas / n;
  out5[3] = s.occ_smem / n;
  out5[4] = s.occ_queued / n;
  out8[5] = (double)s.stop_mem;
  out8[6] = (double)s.stop_smem;
  out8[7] = (double)s.stop_ctas;
  out10[8] = s.rounds ? s.bal_sum / (double)s.rounds : 0.0;
  out10[9] = s.gap_s;
  return gb::OK;
}

const char *gb_server_error(const gb_server *srv) {
  if (!srv)
    return "";
  return srv->s.last_error.c_str();
}

}  // extern "C"
