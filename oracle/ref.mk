# Builds the reference implementation's pybind11 module from its own sources
# where they lie (read-only), with the reference's compile flags plus
# -ffp-contract=off. Output goes only to oracle/_ref/ (git-ignored).
#
#   make -f oracle/ref.mk            # run from the repository root
#
# The reference tree is only available in the development container; on
# machines without it this recipe is skipped by the build helper.
REF      ?= $(or $(FFG_REFERENCE_SRC),/root/reference)
PYTHON   ?= python3
OUT      := oracle/_ref
EXT      := $(shell $(PYTHON) -c "import sysconfig;print(sysconfig.get_config_var('EXT_SUFFIX'))")
PYBIND   := $(shell $(PYTHON) -m pybind11 --includes 2>/dev/null)
CXXFLAGS := -O3 -std=c++20 -shared -fPIC -fopenmp -DFF_OPENMP -DFF_VERSION='"ref"' \
            -ffp-contract=off -w

all: $(OUT)/ffcore$(EXT)

$(OUT)/ffcore$(EXT): $(wildcard $(REF)/src/*.h $(REF)/src/pauli/*.h) $(REF)/src/python_bind.cpp
	mkdir -p $(OUT)
	$(CXX) $(CXXFLAGS) -I$(REF)/src -I$(REF)/src/hashmap $(PYBIND) \
	    $(REF)/src/python_bind.cpp -o $@

.PHONY: all
