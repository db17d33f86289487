# Compiles the reference's own transform sources, unmodified, from the reference tree into
# oracle/_ref/libfdcl_ref.so, against the Eigen-API subset in ref_shim/ (the reference's Eigen
# submodule is not vendored).  Test infrastructure: it pins the restated oracle to the reference's
# code.  Usage: make -f oracle/ref.mk REF=<reference root>
REF ?= /root/reference
CXX ?= g++
HERE := $(dir $(abspath $(lastword $(MAKEFILE_LIST))))
OUT := $(HERE)_ref
# -ffp-contract=off as for the oracle: no fused multiply-add, so both round alike on any host
CXXFLAGS ?= -O2 -fPIC -fopenmp -std=c++14 -ffp-contract=off -w
SRCS := fdcl_FFTSO3.cpp fdcl_FFTS2.cpp fdcl_FFTSO3_matrix.cpp fdcl_FFTS2_matrix.cpp \
        fdcl_Clebsch_Gordon.cpp fdcl_tictoc.cpp fdcl_omp_thread.cpp misc_matrix_func.cpp
OBJS := $(addprefix $(OUT)/,$(SRCS:.cpp=.o))
INC := -I$(HERE)ref_shim -I$(REF)/include

all: $(OUT)/libfdcl_ref.so

# exits non-zero when the reference tree is not there
check:
	@test -f $(REF)/src/fdcl_FFTSO3.cpp

$(OUT)/%.o: $(REF)/src/%.cpp $(wildcard $(HERE)ref_shim/Eigen/*) $(HERE)ref_shim/unsupported/Eigen/FFT
	@mkdir -p $(OUT)
	$(CXX) $(CXXFLAGS) $(INC) -c $< -o $@

$(OUT)/ref_capi.o: $(HERE)ref_capi.cpp $(wildcard $(HERE)ref_shim/Eigen/*)
	@mkdir -p $(OUT)
	$(CXX) $(CXXFLAGS) $(INC) -c $< -o $@

$(OUT)/libfdcl_ref.so: $(OBJS) $(OUT)/ref_capi.o
	$(CXX) -shared -fopenmp -o $@ $^

clean:
	rm -rf $(OUT)

.PHONY: all check clean
