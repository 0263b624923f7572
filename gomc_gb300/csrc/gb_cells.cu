// CellList::GridAll on the device: exact FP64 PositionToCell per atom, a
// scatter into padded cells, then one CTA per cell sorts its atoms by index
// (the order GetCellListNeighbor gives, src/CellList.cpp:258-285) and writes
// the cell-ordered SoA slots (x, y, z, q as double4_32a; molecule/kind; 32-bit
// fixed-point turns for the mixed form).
#include "gb_box.h"
#include "gb_cells.cuh"

#include <climits>

namespace gb {

__global__ void k_cell_scatter(DevBox b, const double *__restrict__ x,
                               const double *__restrict__ y,
                               const double *__restrict__ z) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b.n_atoms)
    return;
  int c = position_to_cell_fast(b, x[i], y[i], z[i]);
  if (c < 0 || c >= b.ncell) {
    atomicOr(b.err, DERR_BAD_INPUT);
    return;
  }
  int s = atomicAdd(&b.cell_count[c], 1);
  if (s < b.cap)
    b.cell_atom[(size_t)c * b.cap + s] = i;
  else
    atomicOr(b.err, DERR_CELL_OVERFLOW);
}

// One CTA per cell: bitonic sort of the cell's atom indices in shared memory.
__global__ void k_cell_sort_fill(DevBox b, const double *__restrict__ x,
                                 const double *__restrict__ y,
                                 const double *__restrict__ z) {
  extern __shared__ int ids[];
  int c = blockIdx.x;
  int n = b.cell_count[c];
  if (n > b.cap)
    n = b.cap;
  if (threadIdx.x == 0)
    b.cell_count[c] = n;
  int P = 1;
  while (P < n)
    P <<= 1;
  for (int i = threadIdx.x; i < P; i += blockDim.x)
    ids[i] = i < n ? b.cell_atom[(size_t)c * b.cap + i] : INT_MAX;
  __syncthreads();
  for (int k = 2; k <= P; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < P; i += blockDim.x) {
        int l = i ^ j;
        if (l > i) {
          int a = ids[i], bb = ids[l];
          bool up = (i & k) == 0;
          if ((a > bb) == up) {
            ids[i] = bb;
            ids[l] = a;
          }
        }
      }
      __syncthreads();
    }
  for (int s = threadIdx.x; s < n; s += blockDim.x) {
    int a = ids[s];
    cell_write_slot(b, c, s, a, x[a], y[a], z[a]);
  }
}

// CellList::RemoveMol (src/CellList.cpp:81-113): take molecule m's atoms out
// of their cells (the cell's last slot fills each hole); an atom out of the
// grid has atom_cell = -1.  One thread: a molecule has a few atoms.
__global__ void k_cell_remove_mol(DevBox b, int m) {
  for (int a = b.mstart[m]; a < b.mstart[m + 1]; ++a) {
    int c0 = b.atom_cell[a];
    if (c0 < 0)
      continue;
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
    b.atom_cell[a] = -1;
    b.atom_slot[a] = -1;
  }
}

// CellList::AddMol (src/CellList.cpp:115-135): put molecule m's atoms, at
// their current coordinates, into the cells PositionToCell gives.
__global__ void k_cell_add_mol(DevBox b, int m) {
  for (int a = b.mstart[m]; a < b.mstart[m + 1]; ++a) {
    if (b.atom_cell[a] >= 0)
      continue;
    double x = b.x[a], y = b.y[a], z = b.z[a];
    int c = position_to_cell_fast(b, x, y, z);
    if (c < 0 || c >= b.ncell) {
      atomicOr(b.err, DERR_BAD_INPUT);
      return;
    }
    int s = b.cell_count[c];
    if (s >= b.cap) {
      atomicOr(b.err, DERR_CELL_OVERFLOW);
      return;
    }
    b.cell_count[c] = s + 1;
    cell_write_slot(b, c, s, a, x, y, z);
  }
}

int launch_cell_remove_mol(Box &bx, int m) {
  k_cell_remove_mol<<<1, 1, 0, bx.stream>>>(bx.dev, m);
  return bx.CudaCheck(cudaGetLastError(), "cell remove");
}

int launch_cell_add_mol(Box &bx, int m) {
  k_cell_add_mol<<<1, 1, 0, bx.stream>>>(bx.dev, m);
  return bx.CudaCheck(cudaGetLastError(), "cell add");
}

int launch_grid_all(Box &bx, const DevBox &b) {
  cudaStream_t st = bx.stream;
  int rc = bx.CudaCheck(cudaMemsetAsync(b.cell_count, 0, b.ncell * 4, st),
                        "memset");
  if (rc)
    return rc;
  k_cell_scatter<<<(b.n_atoms + 255) / 256, 256, 0, st>>>(b, b.x, b.y, b.z);
  int P = 1;
  while (P < b.cap)
    P <<= 1;
  k_cell_sort_fill<<<b.ncell, 256, P * sizeof(int), st>>>(b, b.x, b.y, b.z);
  return bx.CudaCheck(cudaGetLastError(), "grid kernels");
}

}  // namespace gb
