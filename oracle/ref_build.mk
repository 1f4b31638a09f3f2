# Compiles the NeoPZ reference library sources directly with g++ (the
# reference's own CMake build is not used) into oracle/_ref/libpzref.so, and
# links the fixture harness oracle/ref_harness.cpp against it.  Test
# infrastructure only: the library and the harness write the reference-side
# fixtures under tests/golden/; nothing in the product links them.
#
#   make -f oracle/ref_build.mk REF=<NeoPZ source tree> -j8
#
# Configuration: oracle/ref_include/pz_config.h (double real/state types, no
# optional libraries) and the definitions of the reference's Release builds
# (PZNODEBUG, ZERO_INTERNAL_RESIDU, MAKEINTERNAL).  Sources: every .cpp of the
# library directories, minus those that the reference's own build leaves out
# by default (optional third-party libraries, the plasticity and SBFem
# modules, the sources kept under needrefactor/).
REF ?= /root/reference
HERE := $(patsubst %/,%,$(dir $(lastword $(MAKEFILE_LIST))))
OUT := $(HERE)/_ref
DIRS := PerfUtil Util Common Save Integral Solvers Matrix Topology Geom SpecialMaps Shape Refine External \
        Material Mesh Analysis Post Frontal StrMatrix Pre SubStruct Random Optimization Exception
SRCS := $(shell find $(addprefix $(REF)/,$(DIRS)) -name '*.cpp' -not -path '*/needrefactor/*' \
          -not -path '*/Material/Plasticity/*' -not -name 'TPZSBFem*' -not -name 'TPZBuildSBFem*' \
          -not -name TPZBoostGraph.cpp | sort)
INCDIRS := $(HERE)/ref_include $(shell find $(addprefix $(REF)/,$(DIRS)) -type d | sort)
CXXFLAGS := -std=c++17 -O2 -fPIC -w -include cstdint -DPZNODEBUG -DZERO_INTERNAL_RESIDU -DMAKEINTERNAL \
            $(addprefix -I,$(INCDIRS))
OBJS := $(patsubst $(REF)/%.cpp,$(OUT)/obj/%.o,$(SRCS))

all: $(OUT)/libpzref.so $(OUT)/ref_harness

$(OUT)/obj/%.o: $(REF)/%.cpp
	@mkdir -p $(dir $@)
	g++ $(CXXFLAGS) -c $< -o $@

$(OUT)/libpzref.so: $(OBJS)
	g++ -shared -o $@ $(OBJS) -lpthread -latomic

$(OUT)/ref_harness: $(HERE)/ref_harness.cpp $(HERE)/ref_cases.h $(OUT)/libpzref.so
	g++ $(CXXFLAGS) -o $@ $< -L$(OUT) -lpzref -Wl,-rpath,'$$ORIGIN' -lpthread -latomic

# tests/binding_check.cpp: the NeoPZ-side binding (neopz_gb300/neopz_binding)
# compiled against the reference headers, linked with libpzref and the GPU
# library (neopz_gb300/_build, made by the package build)
ROOT := $(HERE)/..
GPZ_BUILD := $(ROOT)/neopz_gb300/_build
$(OUT)/binding_check: $(ROOT)/tests/binding_check.cpp $(ROOT)/tests/grid_cases.h $(HERE)/ref_cases.h \
    $(ROOT)/neopz_gb300/neopz_binding/gpz_neopz.h $(ROOT)/include/gpz.h $(OUT)/libpzref.so
	g++ $(CXXFLAGS) -I$(HERE) -I$(ROOT)/include -I$(ROOT)/neopz_gb300/host -I$(ROOT)/neopz_gb300/neopz_binding \
	  -o $@ $< -L$(OUT) -lpzref -L$(GPZ_BUILD) -lgpzhost -lgpz -Wl,-rpath,'$$ORIGIN' -Wl,-rpath,$(abspath $(GPZ_BUILD)) \
	  -lpthread -latomic

binding: $(OUT)/binding_check

.PHONY: all binding
