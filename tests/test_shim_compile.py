"""The reference-side shim compiles against the reference's own headers and
links against its objects and the GB300 library (no GPU needed).

gomc_gb300/shim/EwaldGB300.h overrides the virtual Ewald interface
(src/Ewald.h:49-179) with `override` on every method, so a signature that
drifts from the reference fails to compile; gomc_gb300/shim/
CalculateEnergyGB300.h wraps the non-virtual CalculateEnergy / CellList calls
with the reference's argument types.  Flags and include paths are those of
oracle/ref.mk; the reference objects are the ones it built.  Skipped where
the reference sources or those objects are absent (the GPU machine has neither).
"""
import glob
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("GOMC_REFERENCE", "/root/reference")
OBJ = os.path.join(ROOT, "oracle", "_ref", "obj_ens1")
GEN = os.path.join(ROOT, "oracle", "_ref", "gen")
LIB = os.path.join(ROOT, "gomc_gb300", "_build", "libgomc_gb300.so")

SRC = r"""
#include "CalculateEnergyGB300.h"
#include "EwaldGB300.h"

// instantiate the shim so that every override and every C ABI call it makes
// is emitted and linked
EwaldGB300 *make_ewald(StaticVals &stat, System &sys, gb_box *const *boxes) {
  return new EwaldGB300(stat, sys, boxes, 1);
}
bool molecule_inter(gb_box *b, Intermolecular &lj, Intermolecular &re,
                    XYZArray const &c, uint m) {
  return gb300::MoleculeInter(b, lj, re, c, m);
}
SystemPotential box_inter(gb_box *b, SystemPotential p, XYZArray const &c,
                          BoxDimensions const &ax) {
  return gb300::BoxInter(b, p, c, ax, 0);
}
SystemPotential box_force(gb_box *b, SystemPotential p, XYZArray const &c,
                          XYZArray &af, XYZArray &mf) {
  return gb300::BoxForce(b, p, c, af, mf, 0);
}
void particle_inter(gb_box *b, double *en, double *re, XYZArray const &t,
                    bool *ov, uint part, uint mol, uint n) {
  gb300::ParticleInter(b, en, re, t, ov, part, mol, n);
}
void single_mol(gb_box *b, Energy &o, Energy &n, uint m) {
  gb300::SingleMoleculeInter(b, o, n, 1.0, 0.5, 1.0, 0.5, m);
}
void cells(gb_box *b, int m) {
  gb300::RemoveMol(b, m);
  gb300::AddMol(b, m);
}
int main() { return 0; }
"""


def test_shim_compiles_and_links(tmp_path):
    if not os.path.isdir(os.path.join(REF, "src")):
        pytest.skip("reference sources not present")
    objs = [o for o in glob.glob(os.path.join(OBJ, "*.o"))
            if os.path.basename(o) not in ("main.o", "ref_probe.o")]
    if not objs or not os.path.exists(os.path.join(GEN, "GOMC_Config.h")):
        pytest.skip("reference objects not built (build() builds them)")
    if not os.path.exists(LIB) or shutil.which("g++") is None:
        pytest.skip("library or compiler missing")
    src = tmp_path / "shim_check.cpp"
    src.write_text(SRC)
    inc = ["-I" + GEN, "-I" + os.path.join(REF, "lib"),
           "-I" + os.path.join(REF, "src"),
           "-I" + os.path.join(REF, "src", "cbmc"),
           "-I" + os.path.join(REF, "src", "moves"),
           "-I" + os.path.join(REF, "src", "GPU"),
           "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(ROOT, "gomc_gb300", "shim")]
    obj = tmp_path / "shim_check.o"
    p = subprocess.run(["g++", "-O1", "-std=c++17", "-w", "-DENSEMBLE=1"] +
                       inc + ["-c", str(src), "-o", str(obj)],
                       capture_output=True, text=True)
    assert p.returncode == 0, p.stderr[-4000:]
    exe = tmp_path / "shim_check"
    cuda_lib = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"),
                            "lib64")
    p = subprocess.run(["g++", "-o", str(exe), str(obj)] + sorted(objs) +
                       ["-L" + os.path.dirname(LIB), "-lgomc_gb300",
                        "-L" + cuda_lib, "-lcudart",
                        "-Wl,--allow-multiple-definition"],
                       capture_output=True, text=True)
    assert p.returncode == 0, p.stderr[-4000:]
