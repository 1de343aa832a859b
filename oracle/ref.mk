# Builds the reference executor `graph_mining_system` from the reference's own
# sources, where they lie, into oracle/_ref/ (never committed: listed in
# .gitignore).  This is the checker's ground truth, not the product.
#
#   make -f oracle/ref.mk REF=/path/to/subgraph-enumeration -j8
#
# nauty (utility/automorphism) and GLPK 4.55 (utility/td/glpk-4.55) are
# compiled from their vendored C sources with the pre-configured headers that
# ship in the tree (nauty.h, glpk-4.55/config.h); the reference's CMake and
# autotools builds are not run.  On an x86 host the reference's AVX2
# intersection path is used; on any other host -D__APPLE__ selects its scalar
# path (identical counts).
ifndef REF
  $(error set REF to the reference checkout, e.g. make -f oracle/ref.mk REF=<path>)
endif
OUT    ?= oracle/_ref
OBJ    ?= /tmp/sge_ref_obj
ARCH   := $(shell uname -m)
ifeq ($(ARCH),x86_64)
  ISA  := -mavx2 -mpopcnt -mbmi -mbmi2 -mfma
else
  ISA  := -D__APPLE__
endif
CXX    ?= g++
CC     ?= gcc
CXXFLAGS := -O3 -std=c++17 -fopenmp -include cstdint $(ISA) -w \
  -I$(REF)/config -I$(REF)/utility -I$(REF)/relation -I$(REF)/plan \
  -I$(REF)/matching -I$(REF)/utility/automorphism -I$(REF)/utility/td \
  -I$(REF)/utility/td/glpk-4.55/src
GLPK   := $(REF)/utility/td/glpk-4.55
GLPKINC := -I$(GLPK) -I$(GLPK)/src $(addprefix -I$(GLPK)/src/,amd bflib cglib colamd env minisat misc proxy zlib)
CFLAGS_GLPK := -O2 -w -DHAVE_CONFIG_H $(GLPKINC)
CFLAGS_NAUTY := -O3 -w -I$(REF)/utility/automorphism

CXX_SRC := main.cpp matching/join.cpp matching/parallel.cpp \
  plan/decomposition.cpp plan/estimator.cpp plan/optimizer.cpp plan/subset_structure.cpp plan/all_td.cpp \
  relation/candidate_space.cpp relation/labeled_graph.cpp relation/relation.cpp relation/graph.cpp \
  utility/command_parser.cpp utility/utils.cpp utility/command.cpp utility/compute_set_intersection.cpp utility/clique.cpp \
  utility/td/hypergraph.cpp utility/td/preprocessing.cpp utility/td/td.cpp utility/td/twbound.cpp utility/td/SCsolver.cpp
NAUTY_SRC := nauty.c nautil.c nausparse.c naugraph.c schreier.c naurng.c traces.c gtools.c naututil.c \
  nautinv.c gutil1.c gutil2.c gtnauty.c naugroup.c
GLPK_SRC := $(filter-out src/proxy/main.c,$(patsubst $(GLPK)/%,%,$(wildcard $(GLPK)/src/*.c $(GLPK)/src/*/*.c)))

CXX_OBJ   := $(addprefix $(OBJ)/ref/,$(CXX_SRC:.cpp=.o))
NAUTY_OBJ := $(addprefix $(OBJ)/nauty/,$(NAUTY_SRC:.c=.o))
GLPK_OBJ  := $(addprefix $(OBJ)/glpk/,$(GLPK_SRC:.c=.o))

all: $(OUT)/graph_mining_system

$(OUT)/graph_mining_system: $(CXX_OBJ) $(NAUTY_OBJ) $(GLPK_OBJ)
	@mkdir -p $(OUT)
	$(CXX) -fopenmp -o $@ $(CXX_OBJ) $(NAUTY_OBJ) $(GLPK_OBJ) -lm

$(OBJ)/ref/%.o: $(REF)/%.cpp
	@mkdir -p $(dir $@)
	$(CXX) $(CXXFLAGS) -c $< -o $@

$(OBJ)/nauty/%.o: $(REF)/utility/automorphism/%.c
	@mkdir -p $(dir $@)
	$(CC) $(CFLAGS_NAUTY) -c $< -o $@

$(OBJ)/glpk/%.o: $(GLPK)/%.c
	@mkdir -p $(dir $@)
	$(CC) $(CFLAGS_GLPK) -c $< -o $@

clean:
	rm -rf $(OUT)

.PHONY: all clean
