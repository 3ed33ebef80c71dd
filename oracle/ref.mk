# Compiles the reference's own sources for the hot path, straight from the
# read-only reference tree, into oracle/_ref/ (git-ignored).  Used only to pin
# the oracle restatement and to generate golden vectors.
#
#   make -f oracle/ref.mk REF=<path of the reference tree>
#
# Flags: -O2 without -ffast-math and with -ffp-contract=off, matching
# oracle/Makefile, so that FP64 results can be compared bit for bit.  (The
# reference's own Makefiles add -march=native -ffast-math, which lets the
# compiler reassociate; those binaries are used for timing only.)
ifndef REF
$(error REF=<path of the reference tree> is required)
endif
HERE := $(dir $(abspath $(lastword $(MAKEFILE_LIST))))
OUT := $(HERE)_ref
CC ?= gcc
CXX ?= g++
FLAGS = -O2 -D_GNU_SOURCE -ffp-contract=off -fno-fast-math -fPIC
GOLDNC := $(REF)/origin/GoldenC/src
FANSRC := $(REF)/helical/rebin/src

MSBEAM := $(REF)/msbeam/CPU_OpenMP/src

CONESRC := $(REF)/industry3d/src
CONEINC := $(REF)/industry3d/include

all: $(OUT)/libgoldnc_ref.so $(OUT)/libfan_ref.so $(OUT)/goldnc_fast $(OUT)/libmsbeam_ref.so $(OUT)/libcone_ref.so

$(OUT):
	mkdir -p $(OUT)

# GoldenC main.c + proj.c as a library; main() renamed so the solver entry
# points (minimize_in_IMAGE_variable, ...) can be driven from tests.
$(OUT)/libgoldnc_ref.so: $(GOLDNC)/main.c $(GOLDNC)/proj.c | $(OUT)
	$(CC) $(FLAGS) -std=c99 -w -I$(GOLDNC) -Dmain=goldnc_ref_main -shared -o $@ $(GOLDNC)/main.c $(GOLDNC)/proj.c -lm

# helical/rebin tracing.cpp with small stubs for the globals it reads.
$(OUT)/libfan_ref.so: $(FANSRC)/tracing.cpp $(HERE)ref_shims/fan_ref_shim.cpp | $(OUT)
	$(CXX) $(FLAGS) -std=c++14 -w -I$(FANSRC) -shared -o $@ $(FANSRC)/tracing.cpp $(HERE)ref_shims/fan_ref_shim.cpp -lm

# GoldenC with the reference's own optimisation flags (timing comparator only).
$(OUT)/goldnc_fast: $(GOLDNC)/main.c $(GOLDNC)/proj.c | $(OUT)
	$(CC) -O3 -std=c99 -D_GNU_SOURCE -w -funroll-all-loops -ffast-math -I$(GOLDNC) -Dmain=goldnc_ref_main -shared -fPIC -o $(OUT)/libgoldnc_fast.so $(GOLDNC)/main.c $(GOLDNC)/proj.c -lm && touch $@

# msbeam/CPU_OpenMP (main.c, proj.c, utility.c) with main() renamed; its
# globals f, v, g and MSbeam() are driven from tests.
$(OUT)/libmsbeam_ref.so: $(MSBEAM)/main.c $(MSBEAM)/proj.c $(MSBEAM)/utility.c | $(OUT)
	$(CC) $(FLAGS) -std=gnu99 -w -fopenmp -I$(MSBEAM) -Dmain=msbeam_ref_main -shared -o $@ \
	    $(MSBEAM)/main.c $(MSBEAM)/proj.c $(MSBEAM)/utility.c -lm

# industry3d's cone geometry and 3D tracer (tracing.cpp, utility.cpp unchanged;
# utility.cpp includes a Boost header it does not use, stood in by an empty one)
$(OUT)/libcone_ref.so: $(CONESRC)/tracing.cpp $(CONESRC)/utility.cpp $(HERE)ref_shims/cone_ref_shim.cpp | $(OUT)
	$(CXX) $(FLAGS) -std=c++14 -w -I$(CONEINC) -I$(HERE)ref_shims/include -shared -o $@ \
	    $(CONESRC)/tracing.cpp $(CONESRC)/utility.cpp $(HERE)ref_shims/cone_ref_shim.cpp -lm

clean:
	rm -rf $(OUT)
.PHONY: all clean
