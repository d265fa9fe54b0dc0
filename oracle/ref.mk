# Builds the reference MCAC (giraldeau/MCAC) from its own sources, where they
# lie, into oracle/_ref/ -- test infrastructure only (the oracle), never part
# of the product. The reference's CMake build needs network fetches (GSL,
# inipp, libunwind, Xdmf, HDF5), so this recipe compiles the translation units
# directly with three small shims from oracle/ref_shims/:
#   * inipp.h   -- INI reader with upstream inipp's extract() semantics
#   * gsl/gsl   -- empty (gsl::at is only used by the HDF5 writer)
#   * backtrace_stub.cpp -- replaces src/exceptions.cpp (libunwind)
# Left out: src/arvo, src/sbl (optional volume back-ends, OFF by default) and
# the HDF5 writer (compiled without WITH_HDF5, i.e. WITH_IO=OFF).
# FP contraction is pinned off so results do not depend on FMA availability;
# DEBUG_MCAC is not defined (it would force seed 0).
#
# Usage: make -f oracle/ref.mk REF=/path/to/reference   (run from the repo root)
ifndef REF
$(error REF must name the reference's source directory)
endif
OUT := oracle/_ref
CXX ?= g++
CXXFLAGS := -std=gnu++17 -O2 -frounding-math -ffp-contract=off -fopenmp -w \
  -I$(REF)/include -Ioracle/ref_shims \
  -include array -include string -include vector -include cmath -include memory \
  -include limits -include tuple -include numeric -include unordered_map -include map \
  -include set -include algorithm -include functional

SRCS := $(shell find $(REF)/src -name '*.cpp' -not -path '*/arvo/*' -not -path '*/sbl/*' \
          -not -name exceptions.cpp -not -name main.cpp | sort)
OBJS := $(patsubst $(REF)/src/%.cpp,$(OUT)/obj/%.o,$(SRCS)) $(OUT)/obj/backtrace_stub.o

all: $(OUT)/MCAC $(OUT)/mcac_ref_harness

$(OUT)/obj/%.o: $(REF)/src/%.cpp
	@mkdir -p $(dir $@)
	$(CXX) $(CXXFLAGS) -c $< -o $@

$(OUT)/obj/backtrace_stub.o: oracle/ref_shims/backtrace_stub.cpp
	@mkdir -p $(dir $@)
	$(CXX) $(CXXFLAGS) -c $< -o $@

$(OUT)/libmcac_ref.a: $(OBJS)
	ar rcs $@ $^

$(OUT)/MCAC: $(REF)/src/main.cpp $(OUT)/libmcac_ref.a
	$(CXX) $(CXXFLAGS) $< $(OUT)/libmcac_ref.a -o $@ -lstdc++fs

$(OUT)/mcac_ref_harness: oracle/ref_harness.cpp $(OUT)/libmcac_ref.a
	$(CXX) $(CXXFLAGS) $< $(OUT)/libmcac_ref.a -o $@ -lstdc++fs

.PHONY: all
