# Builds the reference implementation's pybind11 module from its own sources,
# with the reference's compile flags plus -ffp-contract=off.  Two targets:
#
#   make -f oracle/ref.mk            # from the sources where they lie (read-only),
#                                    # into oracle/_ref/ (git-ignored): the module
#                                    # that regenerates the golden fixtures
#   make -f oracle/ref.mk install    # from the copy staged by oracle/stage_reference.py
#                                    # in baseline/_ref/_src, into baseline/_ref/fastfermion/
#                                    # (git-ignored; on machines without the reference
#                                    # tree, e.g. the GPU hosts)
#
# Run from the repository root.  The build helper skips whichever target has
# no sources on the machine.
REF      ?= $(or $(FFG_REFERENCE_SRC),/root/reference)
PYTHON   ?= python3
OUT      := oracle/_ref
STAGE    := baseline/_ref
EXT      := $(shell $(PYTHON) -c "import sysconfig;print(sysconfig.get_config_var('EXT_SUFFIX'))")
PYINC    := -I$(shell $(PYTHON) -c "import sysconfig;print(sysconfig.get_paths()['include'])")
PYBIND   := $(shell $(PYTHON) -m pybind11 --includes 2>/dev/null)
CXXFLAGS := -O3 -std=c++20 -shared -fPIC -fopenmp -DFF_OPENMP -DFF_VERSION='"ref"' \
            -ffp-contract=off -w

all: $(OUT)/ffcore$(EXT)

$(OUT)/ffcore$(EXT): $(wildcard $(REF)/src/*.h $(REF)/src/pauli/*.h) $(REF)/src/python_bind.cpp
	mkdir -p $(OUT)
	$(CXX) $(CXXFLAGS) -I$(REF)/src -I$(REF)/src/hashmap $(PYBIND) \
	    $(REF)/src/python_bind.cpp -o $@

install: $(STAGE)/fastfermion/ffcore$(EXT)

$(STAGE)/fastfermion/ffcore$(EXT): $(wildcard $(STAGE)/_src/src/*.h $(STAGE)/_src/src/pauli/*.h) \
                                   $(STAGE)/_src/src/python_bind.cpp
	$(CXX) $(CXXFLAGS) -I$(STAGE)/_src/src -I$(STAGE)/_src/src/hashmap -I$(STAGE)/_pybind11/include \
	    $(PYINC) $(STAGE)/_src/src/python_bind.cpp -o $@.tmp && mv $@.tmp $@

.PHONY: all install
