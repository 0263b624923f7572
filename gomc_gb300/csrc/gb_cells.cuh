// Device-side cell-grid helpers shared by the rebuild kernels and the
// Monte Carlo commit path.
#pragma once

#include "gb_internal.h"

namespace gb {

__device__ __forceinline__ int pack_meta(int mol, int kind) {
  return (mol << 4) | kind;
}
__device__ __forceinline__ int meta_mol(int meta) { return meta >> 4; }
__device__ __forceinline__ int meta_kind(int meta) { return meta & 15; }

// Write the packed slot data of atom `a` at (cell, slot); `tur`, when
// given, holds the position's fixed-point turns (to_turns of x, y, z).
__device__ __forceinline__ void cell_write_slot(const DevBox &b, int cell,
                                                int slot, int a, double x,
                                                double y, double z,
                                                const uint32_t *tur = nullptr) {
  size_t s = (size_t)cell * b.cap + slot;
  double q = b.q[a];
  b.cell_atom[s] = a;
  b.cell_pos[s] = make_double4_32a(x, y, z, q);
  b.cell_meta[s] = pack_meta(b.mol[a], b.kind[a]);
  double qs = q * SQRT_QQ_FACT;
  float qsf = (float)qs;
  if (tur)
    b.cell_fix[s] = make_uint4(tur[0], tur[1], tur[2], __float_as_uint(qsf));
  else
    b.cell_fix[s] = make_uint4(to_turns(x, b.invL[0]), to_turns(y, b.invL[1]),
                               to_turns(z, b.invL[2]), __float_as_uint(qsf));
  b.cell_qlo[s] = (float)(qs - (double)qsf);
  b.atom_cell[a] = cell;
  b.atom_slot[a] = slot;
}

// Move atom `a` to new coordinates (already wrapped), relinking it between
// cells the way RemoveMol + AddMol do (src/CellList.cpp:81-135): the set of
// atoms per cell changes exactly as in the reference; the slot order inside a
// cell is this grid's own (swap-remove, append).  Single-thread use.
__device__ __forceinline__ bool cell_move_atom(const DevBox &b, int a, double x,
                                               double y, double z, int c1,
                                               const uint32_t *tur = nullptr) {
  int c0 = b.atom_cell[a];
  if (c0 == c1) {
    cell_write_slot(b, c0, b.atom_slot[a], a, x, y, z, tur);
    return true;
  }
  if (b.cell_count[c1] >= b.cap) {
    atomicOr(b.err, DERR_CELL_OVERFLOW);
    return false;
  }
  // remove from c0: the last slot fills the hole
  int s0 = b.atom_slot[a];
  int last = b.cell_count[c0] - 1;
  if (s0 != last) {
    size_t from = (size_t)c0 * b.cap + last, to = (size_t)c0 * b.cap + s0;
    int moved = b.cell_atom[from];
    b.cell_atom[to] = moved;
    b.cell_pos[to] = b.cell_pos[from];
    b.cell_meta[to] = b.cell_meta[from];
    b.cell_fix[to] = b.cell_fix[from];
    b.cell_qlo[to] = b.cell_qlo[from];
    b.atom_slot[moved] = s0;
  }
  b.cell_count[c0] = last;
  int s1 = b.cell_count[c1];
  b.cell_count[c1] = s1 + 1;
  cell_write_slot(b, c1, s1, a, x, y, z, tur);
  return true;
}

}  // namespace gb
