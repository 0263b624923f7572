// The reference's checkpoint file, so that a run can hand its Monte Carlo
// state to or take it from a stock GOMC run.
//
// GOMC writes `Checkpoint` (src/Checkpoint.h:27-169) through a cereal binary
// archive (CheckpointOutput::saveCheckpointFile,
// src/CheckpointOutput.cpp:55-90): the class version (uint32, 0), then the
// members in Checkpoint::serialize order -- the version string (char[5]),
// the step and the true step (uint64), the MT19937 save array (uint32[625]:
// the state and `left`), seedLocation / seedLeft / seedValue (uint32), the
// move-setting vectors (scale, acceptPercent as
// vector<vector<vector<double>>> [box][move][kind]; accepted, tries,
// tempAccepted, tempTries as the same of uint32; the MultiParticle counters
// as vector<vector<uint32>> [box][type]; mp_t_max, mp_r_max as
// vector<double>; isSingleMoveAccepted as vector<bool>, one byte per
// element) -- and after them the molecule start vectors, the molecule lookup,
// the molecule setup and the PDB atom records, then the lookup's raw arrays.
// cereal writes every vector as its size (uint64) followed by its elements,
// little-endian.
//
// This file reads the fields up to isSingleMoveAccepted, and writes a
// checkpoint as a copy of a template checkpoint of the same system (which
// carries the records this library does not hold: molecule setup, PDB
// atoms, lookup) with those fields replaced.
#include "gomc_gb300.h"
#include "gb_box.h"
#include "gb_mc.h"

#include <cstring>
#include <vector>

namespace gb {

namespace {

// Bounds-checked reader of the archive's bytes.
struct In {
  const uint8_t *p;
  size_t n, off = 0;
  bool ok = true;
  void raw(void *dst, size_t k) {
    if (!ok || k > n - off) {
      ok = false;
      std::memset(dst, 0, k);
      return;
    }
    std::memcpy(dst, p + off, k);
    off += k;
  }
  template <class T> T get() {
    T v;
    raw(&v, sizeof(T));
    return v;
  }
  // a vector size, bounded by what the rest of the archive could hold
  size_t size(size_t elem) {
    uint64_t s = get<uint64_t>();
    if (!ok || (elem > 0 && s > (n - off) / elem)) {
      ok = false;
      return 0;
    }
    return (size_t)s;
  }
};

struct Out {
  std::vector<uint8_t> v;
  void raw(const void *src, size_t k) {
    const uint8_t *s = (const uint8_t *)src;
    v.insert(v.end(), s, s + k);
  }
  template <class T> void put(T x) { raw(&x, sizeof(T)); }
};

template <class T> using V1 = std::vector<T>;
template <class T> using V2 = std::vector<std::vector<T>>;
template <class T> using V3 = std::vector<std::vector<std::vector<T>>>;

template <class T> void rd(In &in, V1<T> &v) {
  v.resize(in.size(sizeof(T)));
  if (!v.empty())
    in.raw(v.data(), v.size() * sizeof(T));
}
template <class T> void rd(In &in, V2<T> &v) {
  v.resize(in.size(8));
  for (auto &x : v)
    rd(in, x);
}
template <class T> void rd(In &in, V3<T> &v) {
  v.resize(in.size(8));
  for (auto &x : v)
    rd(in, x);
}
template <class T> void wr(Out &o, const V1<T> &v) {
  o.put<uint64_t>(v.size());
  if (!v.empty())
    o.raw(v.data(), v.size() * sizeof(T));
}
template <class T> void wr(Out &o, const V2<T> &v) {
  o.put<uint64_t>(v.size());
  for (auto &x : v)
    wr(o, x);
}
template <class T> void wr(Out &o, const V3<T> &v) {
  o.put<uint64_t>(v.size());
  for (auto &x : v)
    wr(o, x);
}

// The Checkpoint members this file handles, in serialization order.
struct Prefix {
  uint32_t class_version;
  char version[5];
  uint64_t step, true_step;
  uint32_t save[625];
  uint32_t location, left, seed;
  V3<double> scale, accept_percent;
  V3<uint32_t> accepted, tries, temp_accepted, temp_tries;
  V2<uint32_t> mp_tries, mp_accepted, mp_interval_accepted, mp_interval_tries;
  V1<double> mp_t_max, mp_r_max;
  V1<uint8_t> single;  // vector<bool>: one byte per element
  size_t end;          // bytes up to and including `single`
};

bool read_prefix(const void *buf, int64_t bytes, Prefix &P) {
  if (!buf || bytes <= 0)
    return false;
  In in{(const uint8_t *)buf, (size_t)bytes};
  P.class_version = in.get<uint32_t>();
  in.raw(P.version, 5);
  P.step = in.get<uint64_t>();
  P.true_step = in.get<uint64_t>();
  in.raw(P.save, sizeof P.save);
  P.location = in.get<uint32_t>();
  P.left = in.get<uint32_t>();
  P.seed = in.get<uint32_t>();
  rd(in, P.scale);
  rd(in, P.accept_percent);
  rd(in, P.accepted);
  rd(in, P.tries);
  rd(in, P.temp_accepted);
  rd(in, P.temp_tries);
  rd(in, P.mp_tries);
  rd(in, P.mp_accepted);
  rd(in, P.mp_interval_accepted);
  rd(in, P.mp_interval_tries);
  rd(in, P.mp_t_max);
  rd(in, P.mp_r_max);
  P.single.resize(in.size(1));
  if (!P.single.empty())
    in.raw(P.single.data(), P.single.size());
  P.end = in.off;
  return in.ok;
}

void write_prefix(const Prefix &P, Out &o) {
  o.put(P.class_version);
  o.raw(P.version, 5);
  o.put(P.step);
  o.put(P.true_step);
  o.raw(P.save, sizeof P.save);
  o.put(P.location);
  o.put(P.left);
  o.put(P.seed);
  wr(o, P.scale);
  wr(o, P.accept_percent);
  wr(o, P.accepted);
  wr(o, P.tries);
  wr(o, P.temp_accepted);
  wr(o, P.temp_tries);
  wr(o, P.mp_tries);
  wr(o, P.mp_accepted);
  wr(o, P.mp_interval_accepted);
  wr(o, P.mp_interval_tries);
  wr(o, P.mp_t_max);
  wr(o, P.mp_r_max);
  o.put<uint64_t>(P.single.size());
  if (!P.single.empty())
    o.raw(P.single.data(), P.single.size());
}

// Every [box][move][kind] vector has the same shape, every [box][type]
// vector the same box count, and the shape fits the C structure.
bool shape_ok(const Prefix &P) {
  const size_t nb = P.scale.size();
  if (nb == 0 || nb > GB_CHK_BOXES)
    return false;
  const size_t nm = P.scale[0].size();
  if (nm == 0 || nm > GB_CHK_MOVES)
    return false;
  const size_t nk = P.scale[0][0].size();
  if (nk == 0)
    return false;
  auto same3d = [&](const auto &v) {
    if (v.size() != nb)
      return false;
    for (auto &b : v) {
      if (b.size() != nm)
        return false;
      for (auto &m : b)
        if (m.size() != nk)
          return false;
    }
    return true;
  };
  auto same2 = [&](const auto &v) {
    if (v.size() != nb)
      return false;
    for (auto &b : v)
      if (b.size() > GB_CHK_MP)
        return false;
    return true;
  };
  return same3d(P.scale) && same3d(P.accept_percent) &&
         same3d(P.accepted) && same3d(P.tries) && same3d(P.temp_accepted) &&
         same3d(P.temp_tries) && same2(P.mp_tries) && same2(P.mp_accepted) &&
         same2(P.mp_interval_accepted) && same2(P.mp_interval_tries) &&
         P.mp_t_max.size() == nb && P.mp_r_max.size() == nb &&
         P.single.size() <= GB_CHK_BOXES;
}

void to_c(const Prefix &P, gb_gomc_chk *c) {
  std::memset(c, 0, sizeof *c);
  c->step = P.step;
  c->true_step = P.true_step;
  std::memcpy(c->mt_state, P.save, sizeof c->mt_state);
  c->mt_left = P.save[624];
  c->seed_location = P.location;
  c->seed_left = P.left;
  c->seed_value = P.seed;
  c->n_box = (int32_t)P.scale.size();
  c->n_move = (int32_t)P.scale[0].size();
  c->n_kind = (int32_t)P.scale[0][0].size();
  for (int b = 0; b < c->n_box; ++b) {
    for (int m = 0; m < c->n_move; ++m) {
      c->scale[b][m] = P.scale[b][m][0];
      c->accept_percent[b][m] = P.accept_percent[b][m][0];
      c->accepted[b][m] = P.accepted[b][m][0];
      c->tries[b][m] = P.tries[b][m][0];
      c->temp_accepted[b][m] = P.temp_accepted[b][m][0];
      c->temp_tries[b][m] = P.temp_tries[b][m][0];
    }
    for (size_t t = 0; t < P.mp_tries[b].size(); ++t) {
      c->mp_tries[b][t] = P.mp_tries[b][t];
      c->mp_accepted[b][t] = P.mp_accepted[b][t];
      c->mp_interval_accepted[b][t] = P.mp_interval_accepted[b][t];
      c->mp_interval_tries[b][t] = P.mp_interval_tries[b][t];
    }
    c->mp_t_max[b] = P.mp_t_max[b];
    c->mp_r_max[b] = P.mp_r_max[b];
  }
  for (size_t b = 0; b < P.single.size(); ++b)
    c->single_move_accepted[b] = P.single[b] != 0;
  c->records_offset = (int64_t)P.end;
}

}  // namespace

int gomc_chk_read(const void *buf, int64_t bytes, gb_gomc_chk *out) {
  Prefix P;
  if (!out || !read_prefix(buf, bytes, P) || !shape_ok(P))
    return ERR_ARG;
  to_c(P, out);
  return OK;
}

int gomc_chk_write(const void *tmpl, int64_t tbytes, const gb_gomc_chk *in,
                   void *out, int64_t cap, int64_t *out_bytes) {
  Prefix P;
  if (!in || !out_bytes || !read_prefix(tmpl, tbytes, P) || !shape_ok(P))
    return ERR_ARG;
  if (in->n_box != (int32_t)P.scale.size() ||
      in->n_move != (int32_t)P.scale[0].size() ||
      in->seed_location + in->seed_left != 624 || in->seed_left > 624 ||
      in->mt_left != in->seed_left)
    return ERR_ARG;
  P.step = in->step;
  P.true_step = in->true_step;
  std::memcpy(P.save, in->mt_state, sizeof in->mt_state);
  P.save[624] = in->mt_left;
  P.location = in->seed_location;
  P.left = in->seed_left;
  P.seed = in->seed_value;
  // kind 0 of every [box][move] entry; the template's other kinds stay
  for (size_t b = 0; b < P.scale.size(); ++b) {
    for (size_t m = 0; m < P.scale[b].size(); ++m) {
      P.scale[b][m][0] = in->scale[b][m];
      P.accept_percent[b][m][0] = in->accept_percent[b][m];
      P.accepted[b][m][0] = in->accepted[b][m];
      P.tries[b][m][0] = in->tries[b][m];
      P.temp_accepted[b][m][0] = in->temp_accepted[b][m];
      P.temp_tries[b][m][0] = in->temp_tries[b][m];
    }
    for (size_t t = 0; t < P.mp_tries[b].size(); ++t) {
      P.mp_tries[b][t] = in->mp_tries[b][t];
      P.mp_accepted[b][t] = in->mp_accepted[b][t];
      P.mp_interval_accepted[b][t] = in->mp_interval_accepted[b][t];
      P.mp_interval_tries[b][t] = in->mp_interval_tries[b][t];
    }
    P.mp_t_max[b] = in->mp_t_max[b];
    P.mp_r_max[b] = in->mp_r_max[b];
  }
  for (size_t b = 0; b < P.single.size(); ++b)
    P.single[b] = in->single_move_accepted[b] ? 1 : 0;
  Out o;
  write_prefix(P, o);
  const size_t rest = (size_t)tbytes - P.end;
  const size_t total = o.v.size() + rest;
  *out_bytes = (int64_t)total;
  if (!out)
    return OK;  // a size query
  if ((int64_t)total > cap)
    return ERR_ARG;
  std::memcpy(out, o.v.data(), o.v.size());
  std::memcpy((uint8_t *)out + o.v.size(), (const uint8_t *)tmpl + P.end,
              rest);
  return OK;
}

// The loop state of box 0, molecule kind 0 (the single kind this library's
// Monte Carlo loop moves), as a checkpoint holds it: step, the move
// stream's MT19937 state, the seed, and the move settings (DISPLACE = 0,
// ROTATE = 1, MULTIPARTICLE = 2 of src/MoveConst.h).
int mc_get_gomc_state(Box &b, gb_gomc_chk *c) {
  if (!b.mc)
    return b.Fail(ERR_STATE, "gb_mc_init has not been called");
  McState &s = *b.mc;
  Settings set;
  int rc = b.CudaCheck(cudaMemcpyAsync(&set, s.d_set, sizeof set,
                                       cudaMemcpyDeviceToHost, b.stream),
                       "download");
  if (rc || (rc = b.Sync()))
    return rc;
  std::memset(c, 0, sizeof *c);
  c->step = (uint64_t)s.next_step;
  c->true_step = (uint64_t)s.next_step;
  int32_t left = 0, next = 0;
  stream_state_at_next(s, c->mt_state, &left, &next);
  c->mt_left = (uint32_t)left;
  c->seed_left = (uint32_t)left;
  c->seed_location = (uint32_t)next;
  c->seed_value = s.params.seed;
  c->n_box = 1;
  c->n_move = 9;  // MOVE_KINDS_TOTAL of the NVT build
  c->n_kind = 1;
  c->scale[0][0] = set.scale[0];
  c->scale[0][1] = set.scale[1];
  for (int m = 0; m < 3; ++m) {
    c->accepted[0][m] = (uint32_t)set.accepted[m];
    c->tries[0][m] = (uint32_t)set.tries[m];
    c->temp_accepted[0][m] = (uint32_t)set.tempAccepted[m];
    c->temp_tries[0][m] = (uint32_t)set.tempTries[m];
    // MoveSettings::Update's running acceptance fraction
    c->accept_percent[0][m] =
        set.tries[m] > 0 ? (double)set.accepted[m] / (double)set.tries[m]
                         : 0.0;
  }
  for (int t = 0; t < 2; ++t) {
    c->mp_tries[0][t] = (uint32_t)set.mp_tries[t];
    c->mp_accepted[0][t] = (uint32_t)set.mp_acc[t];
    c->mp_interval_tries[0][t] = (uint32_t)set.mp_itries[t];
    c->mp_interval_accepted[0][t] = (uint32_t)set.mp_iacc[t];
  }
  c->mp_t_max[0] = set.mp_t_max;
  c->mp_r_max[0] = set.mp_r_max;
  c->single_move_accepted[0] = set.singleMoveAccepted;
  return OK;
}

int mc_set_gomc_state(Box &b, const gb_gomc_chk *c) {
  if (!b.mc)
    return b.Fail(ERR_STATE, "gb_mc_init has not been called");
  if (c->n_box < 1 || c->n_move < 3 || c->n_kind != 1)
    return b.Fail(ERR_UNSUPPORTED,
                  "the loop moves one molecule kind in one box");
  if (c->seed_left > 624 || c->seed_location + c->seed_left != 624 ||
      c->mt_left != c->seed_left)
    return b.Fail(ERR_ARG, "checkpoint random-stream state out of range");
  McState &s = *b.mc;
  Settings set;
  int rc = b.CudaCheck(cudaMemcpyAsync(&set, s.d_set, sizeof set,
                                       cudaMemcpyDeviceToHost, b.stream),
                       "download");
  if (rc || (rc = b.Sync()))
    return rc;
  set.scale[0] = c->scale[0][0];
  set.scale[1] = c->scale[0][1];
  for (int m = 0; m < 3; ++m) {
    set.accepted[m] = c->accepted[0][m];
    set.tries[m] = c->tries[0][m];
    set.tempAccepted[m] = c->temp_accepted[0][m];
    set.tempTries[m] = c->temp_tries[0][m];
  }
  for (int t = 0; t < 2; ++t) {
    set.mp_tries[t] = c->mp_tries[0][t];
    set.mp_acc[t] = c->mp_accepted[0][t];
    set.mp_itries[t] = c->mp_interval_tries[0][t];
    set.mp_iacc[t] = c->mp_interval_accepted[0][t];
  }
  set.mp_t_max = c->mp_t_max[0];
  set.mp_r_max = c->mp_r_max[0];
  set.singleMoveAccepted = c->single_move_accepted[0] != 0;
  if ((rc = b.CudaCheck(cudaMemcpyAsync(s.d_set, &set, sizeof set,
                                        cudaMemcpyHostToDevice, b.stream),
                        "upload")) ||
      (rc = b.Sync()))
    return rc;
  s.stream->mt().Load(c->mt_state, (int32_t)c->seed_left,
                      (int32_t)c->seed_location);
  s.ahead.clear();  // records drawn ahead belong to the old position
  s.ahead_pos = 0;
  s.next_step = (int64_t)c->step;
  return OK;
}

}  // namespace gb
