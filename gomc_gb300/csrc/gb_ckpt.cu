// Checkpoints of a box's dynamic state, so that a run resumes exactly where
// it stopped: the same moves, decisions and coordinates, bit for bit, as a
// run that never stopped.  This is the property the reference's restart
// tests pin (test/src/ConsistentTrajectoryTest.cpp, CheckpointTest.cpp) for
// its own format (src/Checkpoint.h:27-120, cereal binary); this file's
// format is its own, and a checkpoint loads into a box created from the same
// system and configuration.
//
// Saved: coordinates and molecule centres; the cell grid's slot order (the
// FP64 sums run over it); the FP64 structure factors (incrementally updated,
// not recomputable to the last bit); the running energies; and, when the box
// has a Monte Carlo loop, its step, the MT19937 state of the move stream,
// the move settings and the mixed form's drift records.
#include "gomc_gb300.h"
#include "gb_box.h"
#include "gb_cells.cuh"
#include "gb_mc.h"

#include <cstring>
#include <vector>

namespace gb {

namespace {

constexpr char MAGIC[8] = {'G', 'B', 'C', 'K', 'P', 'T', '0', '1'};

struct Header {
  char magic[8];
  int32_t precision, n_atoms, n_mol, K, ncell, cap, has_mc, pad;
  int64_t next_step;
};

struct McBlock {
  uint32_t mt[624];
  int32_t mt_left, mt_next;
  Settings set;
  double drift_max[4], drift_last[4];
  int64_t recomputes;
};

size_t body_bytes(const DevBox &d) {
  size_t N = d.n_atoms, M = d.n_mol, K = d.K, NC = (size_t)d.ncell * d.cap;
  return 8 * (3 * N + 3 * M + 5 + 2 * K) + 4 * (d.ncell + NC);
}

// Rewrite every occupied slot from the atom data, in the slot order the grid
// already holds (cell_count / cell_atom restored).
__global__ void k_cell_refill(DevBox b) {
  size_t NC = (size_t)b.ncell * b.cap;
  for (size_t s = blockIdx.x * (size_t)blockDim.x + threadIdx.x; s < NC;
       s += (size_t)gridDim.x * blockDim.x) {
    int c = (int)(s / b.cap), j = (int)(s % b.cap);
    if (j < b.cell_count[c]) {
      int a = b.cell_atom[s];
      cell_write_slot(b, c, j, a, b.x[a], b.y[a], b.z[a]);
    }
  }
}

}  // namespace

int checkpoint_size(Box &b, int64_t *bytes) {
  *bytes = (int64_t)(sizeof(Header) + body_bytes(b.dev) +
                     (b.mc ? sizeof(McBlock) : 0));
  return OK;
}

int checkpoint_save(Box &b, void *buf, int64_t bytes) {
  int64_t need;
  checkpoint_size(b, &need);
  if (bytes < need)
    return b.Fail(ERR_CAPACITY, "checkpoint buffer too small");
  int rc = b.Sync();
  if (rc)
    return rc;
  const DevBox &d = b.dev;
  unsigned char *p = (unsigned char *)buf;
  Header h;
  std::memcpy(h.magic, MAGIC, 8);
  h.precision = b.cfg.precision;
  h.n_atoms = d.n_atoms;
  h.n_mol = d.n_mol;
  h.K = d.K;
  h.ncell = d.ncell;
  h.cap = d.cap;
  h.has_mc = b.mc ? 1 : 0;
  h.pad = 0;
  h.next_step = b.mc ? b.mc->next_step : 0;
  std::memcpy(p, &h, sizeof h);
  p += sizeof h;
  size_t N = d.n_atoms, M = d.n_mol, K = d.K, NC = (size_t)d.ncell * d.cap;
  struct Part {
    const void *src;
    size_t n;
  } parts[] = {{d.x, 8 * N},        {d.y, 8 * N},        {d.z, 8 * N},
               {d.cx, 8 * M},       {d.cy, 8 * M},       {d.cz, 8 * M},
               {d.energy, 8 * 5},   {d.sumRref, 8 * K},  {d.sumIref, 8 * K},
               {d.cell_count, 4 * (size_t)d.ncell}, {d.cell_atom, 4 * NC}};
  for (const Part &q : parts) {
    if (q.n && (rc = b.CudaCheck(cudaMemcpy(p, q.src, q.n,
                                            cudaMemcpyDeviceToHost),
                                 "checkpoint read")))
      return rc;
    p += q.n;
  }
  if (b.mc) {
    McState &s = *b.mc;
    McBlock m;
    int32_t left = 0, next = 0;
    stream_state_at_next(s, m.mt, &left, &next);
    m.mt_left = left;
    m.mt_next = next;
    if ((rc = b.CudaCheck(cudaMemcpy(&m.set, s.d_set, sizeof(Settings),
                                     cudaMemcpyDeviceToHost),
                          "checkpoint read")))
      return rc;
    for (int i = 0; i < 4; ++i) {
      m.drift_max[i] = s.drift_max[i];
      m.drift_last[i] = s.drift_last[i];
    }
    m.recomputes = s.recomputes;
    std::memcpy(p, &m, sizeof m);
  }
  return OK;
}

int checkpoint_load(Box &b, const void *buf, int64_t bytes) {
  if (bytes < (int64_t)sizeof(Header))
    return b.Fail(ERR_ARG, "checkpoint too short");
  const unsigned char *p = (const unsigned char *)buf;
  Header h;
  std::memcpy(&h, p, sizeof h);
  p += sizeof h;
  const DevBox &d = b.dev;
  if (std::memcmp(h.magic, MAGIC, 8) != 0)
    return b.Fail(ERR_ARG, "not a gomc_gb300 checkpoint");
  if (h.precision != b.cfg.precision || h.n_atoms != d.n_atoms ||
      h.n_mol != d.n_mol || h.K != d.K || h.ncell != d.ncell || h.cap != d.cap)
    return b.Fail(ERR_ARG,
                  "checkpoint was written by a box of another system or "
                  "configuration");
  if (h.has_mc && !b.mc)
    return b.Fail(ERR_STATE,
                  "checkpoint holds Monte Carlo state: call gb_mc_init first");
  int64_t need = (int64_t)(sizeof(Header) + body_bytes(d) +
                           (h.has_mc ? sizeof(McBlock) : 0));
  if (bytes < need)
    return b.Fail(ERR_ARG, "checkpoint truncated");
  // Every check of the buffer comes before the first copy, so a rejected
  // checkpoint leaves the box as it was.
  size_t N = d.n_atoms, M = d.n_mol, K = d.K, NC = (size_t)d.ncell * d.cap;
  const unsigned char *grid = p + 8 * (3 * N + 3 * M + 5 + 2 * K);
  // slot counts must fit the grid, and the occupied slots must hold every
  // atom id of this box exactly once
  std::vector<int32_t> cnt(d.ncell), slot_atom(NC);
  std::memcpy(cnt.data(), grid, 4 * cnt.size());
  std::memcpy(slot_atom.data(), grid + 4 * cnt.size(), 4 * NC);
  for (int32_t c : cnt)
    if (c < 0 || c > d.cap)
      return b.Fail(ERR_ARG, "checkpoint cell counts out of range");
  {
    std::vector<char> seen(N, 0);
    size_t placed = 0;
    for (int c = 0; c < d.ncell; ++c)
      for (int j = 0; j < cnt[c]; ++j) {
        int32_t a = slot_atom[(size_t)c * d.cap + j];
        if (a < 0 || a >= d.n_atoms || seen[a])
          return b.Fail(ERR_ARG, "checkpoint cell slots out of range");
        seen[a] = 1;
        ++placed;
      }
    if (placed != N)
      return b.Fail(ERR_ARG, "checkpoint cell slots do not hold every atom");
  }
  McBlock m;
  if (h.has_mc) {
    std::memcpy(&m, grid + 4 * (cnt.size() + NC), sizeof m);
    // MT19937 position: `left` words remain of the current block of 624
    if (m.mt_left < 0 || m.mt_left > 624 || m.mt_next + m.mt_left != 624)
      return b.Fail(ERR_ARG, "checkpoint random-stream state out of range");
  }
  int rc = b.Sync();
  if (rc)
    return rc;
  struct Part {
    void *dst;
    size_t n;
  } parts[] = {{d.x, 8 * N},        {d.y, 8 * N},        {d.z, 8 * N},
               {d.cx, 8 * M},       {d.cy, 8 * M},       {d.cz, 8 * M},
               {d.energy, 8 * 5},   {d.sumRref, 8 * K},  {d.sumIref, 8 * K},
               {d.cell_count, 4 * (size_t)d.ncell}, {d.cell_atom, 4 * NC}};
  for (const Part &q : parts) {
    if (q.n && (rc = b.CudaCheck(cudaMemcpy(q.dst, p, q.n,
                                            cudaMemcpyHostToDevice),
                                 "checkpoint write")))
      return rc;
    p += q.n;
  }
  if (K && ((rc = b.CudaCheck(cudaMemcpy(d.sumRnew, d.sumRref, 8 * K,
                                         cudaMemcpyDeviceToDevice),
                              "copy")) ||
            (rc = b.CudaCheck(cudaMemcpy(d.sumInew, d.sumIref, 8 * K,
                                         cudaMemcpyDeviceToDevice),
                              "copy"))))
    return rc;
  k_cell_refill<<<b.sm_count * 4, 256, 0, b.stream>>>(b.dev);
  if ((rc = b.CudaCheck(cudaGetLastError(), "cell refill")) ||
      (rc = b.Sync()))
    return rc;
  if (h.has_mc) {
    McState &s = *b.mc;
    s.stream->mt().Load(m.mt, m.mt_left, m.mt_next);
    s.ahead.clear();  // records drawn ahead belong to the old position
    s.ahead_pos = 0;
    s.next_step = h.next_step;
    if ((rc = b.CudaCheck(cudaMemcpy(s.d_set, &m.set, sizeof(Settings),
                                     cudaMemcpyHostToDevice),
                          "checkpoint write")))
      return rc;
    for (int i = 0; i < 4; ++i) {
      s.drift_max[i] = m.drift_max[i];
      s.drift_last[i] = m.drift_last[i];
    }
    s.recomputes = m.recomputes;
  }
  return b.CheckError();
}

}  // namespace gb
