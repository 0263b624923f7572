# Builds the reference GOMC CPU code path from its own sources, in place, with
# a plain g++ command line (no CMake).  Everything it writes goes under
# oracle/_ref/ (git-ignored).  Used only to pin the oracle: the probe program
# (ref_probe.cpp) links the reference objects and dumps FP64 energies, k-vector
# tables, cell-list membership and per-move accept decisions for generated
# fixtures.
#
#   make -f oracle/ref.mk REF=/root/reference -j8
#
# The only generated input is the configuration header that the reference's
# CMake would write from GOMC_Config.h.in (version numbers and the test-accessor
# switch); this recipe writes an equivalent one with GOMC_GTEST=1 so that the
# Simulation getters (src/Simulation.h:25-38) are compiled.  No OpenMP, so the
# reference's reductions run in a fixed order.

REF ?= /root/reference
OUT ?= oracle/_ref
ENSEMBLE ?= 1
TAG := ens$(ENSEMBLE)
OBJ := $(OUT)/obj_$(TAG)
GEN := $(OUT)/gen

CXX ?= g++
CXXFLAGS ?= -O2 -std=c++17 -w
INC := -I$(GEN) -I$(REF)/lib -I$(REF)/src -I$(REF)/src/cbmc -I$(REF)/src/moves -I$(REF)/src/GPU
DEFS := -DENSEMBLE=$(ENSEMBLE)

SRC := BlockOutput BondAdjacencyList BoxDimensions BoxDimensionsNonOrth \
  CalculateEnergy CBMC CellList Checkpoint CheckpointOutput CheckpointSetup \
  ConfigSetup ConsoleOutput Coordinates CPUSide DCDlib EnPartCntSampleOutput \
  Ewald EwaldCached ExtendedSystem ExtendedSystemOutput FFConst FFDihedrals \
  FFParticle FFSetup Forcefield FreeEnergyOutput Geometry HistOutput \
  InputFileReader MoleculeKind MoleculeLookup Molecules MolSetup MoveSettings \
  NoEwald OutConst OutputVars ParallelTemperingPreprocessor \
  ParallelTemperingUtilities PDBOutput PDBSetup PRNGSetup PSFOutput \
  Random123Wrapper Reader Simulation StaticVals System
CBMC := DCCrankShaftAng DCCrankShaftDih DCCyclic DCFreeCycle DCFreeCycleSeed \
  DCFreeHedron DCFreeHedronSeed DCGraph DCHedron DCHedronCycle DCLinear \
  DCLinkedCycle DCLinkedHedron DCOnSphere DCRotateCOM DCRotateOnAtom DCSingle \
  TrialMol
LIBSRC := AlphaNum CircuitFinder FloydWarshallCycle

OBJS := $(addprefix $(OBJ)/src_,$(addsuffix .o,$(SRC))) \
        $(addprefix $(OBJ)/cbmc_,$(addsuffix .o,$(CBMC))) \
        $(addprefix $(OBJ)/lib_,$(addsuffix .o,$(LIBSRC)))

all: $(OUT)/ref_probe_$(TAG) $(OUT)/GOMC_CPU_$(TAG)

$(GEN)/GOMC_Config.h:
	@mkdir -p $(GEN)
	@printf '%s\n' '#define GOMC_VERSION_MAJOR 2' '#define GOMC_VERSION_MINOR 80' \
	  '#define GOMC_GTEST 1' '#define GOMC_GTEST_MPI 0' '#define GOMC_LIB_MPI 0' \
	  '#define GOMC_THREAD_MPI 0' '#define GOMC_MPI (GOMC_LIB_MPI || GOMC_THREAD_MPI)' \
	  '#define MPI_IN_PLACE_EXISTS 0' > $@

$(OBJ)/src_%.o: $(REF)/src/%.cpp $(GEN)/GOMC_Config.h
	@mkdir -p $(OBJ)
	$(CXX) $(CXXFLAGS) $(DEFS) $(INC) -c $< -o $@

$(OBJ)/cbmc_%.o: $(REF)/src/cbmc/%.cpp $(GEN)/GOMC_Config.h
	@mkdir -p $(OBJ)
	$(CXX) $(CXXFLAGS) $(DEFS) $(INC) -c $< -o $@

$(OBJ)/lib_%.o: $(REF)/lib/%.cpp $(GEN)/GOMC_Config.h
	@mkdir -p $(OBJ)
	$(CXX) $(CXXFLAGS) $(DEFS) $(INC) -c $< -o $@

$(OBJ)/main.o: $(REF)/src/Main.cpp $(GEN)/GOMC_Config.h
	@mkdir -p $(OBJ)
	$(CXX) $(CXXFLAGS) $(DEFS) $(INC) -c $< -o $@

$(OBJ)/ref_probe.o: oracle/ref_probe.cpp $(GEN)/GOMC_Config.h
	@mkdir -p $(OBJ)
	$(CXX) $(CXXFLAGS) $(DEFS) $(INC) -c $< -o $@

$(OUT)/ref_probe_$(TAG): $(OBJS) $(OBJ)/ref_probe.o
	$(CXX) -o $@ $^ -Wl,--allow-multiple-definition

$(OUT)/GOMC_CPU_$(TAG): $(OBJS) $(OBJ)/main.o
	$(CXX) -o $@ $^ -Wl,--allow-multiple-definition

.PHONY: all
