# Builds the SG++ reference's own FP64 implementation of the multi-evaluation path from the
# reference sources where they lie (read-only), plus oracle/ref_harness.cpp, into
# oracle/_ref/libsgpp_ref.so. Test infrastructure only: used to pin the oracle restatement and
# to generate the golden fixtures under tests/golden/. Object files go to oracle/_ref/obj/.
#
#   make -f oracle/ref.mk -j8 REF=/path/to/reference
#
# Sources: every base/src translation unit except the OpenCL manager (no OpenCL headers
# exist here), solver/src, the STREAMING operators of the Linear and ModLinear bases, the two
# system-matrix files and the ARFF/CSV readers.
# Quirks needed with g++ 13: -include cstdint -include memory (missing includes in the
# reference headers, e.g. base/src/sgpp/base/grid/storage/hashmap/HashGridPoint.hpp).

# REF: the reference checkout (no default; __graft_entry__.build() passes the one that
# oracle.reference_source() finds)
ifndef REF
$(error set REF=<reference checkout>)
endif
OUT := oracle/_ref
OBJ := $(OUT)/obj

UNAME_M := $(shell uname -m)
ifeq ($(UNAME_M),x86_64)
# the reference's own ARCH=avx512 flags (site_scons/SGppConfigure.py:520-523)
ARCHFLAGS := -mavx512f -mavx512cd -mfma
else
ARCHFLAGS :=
endif

CXX ?= g++
CXXFLAGS := -std=c++17 -O3 -fopenmp -fPIC -w $(ARCHFLAGS) -include cstdint -include memory \
            -I$(REF)/base/src -I$(REF)/solver/src -I$(REF)/datadriven/src

BASE_SRCS := $(shell find $(REF)/base/src -name '*.cpp' -not -path '*/opencl/*' | sort)
SOLVER_SRCS := $(shell find $(REF)/solver/src -name '*.cpp' | sort)
DD := $(REF)/datadriven/src/sgpp/datadriven
DD_SRCS := $(DD)/operation/hash/OperationMultiEvalStreaming/OperationMultiEvalStreaming.cpp \
           $(DD)/operation/hash/OperationMultiEvalStreaming/OperationMultiEvalStreaming_multImpl.cpp \
           $(DD)/operation/hash/OperationMultiEvalStreaming/OperationMultiEvalStreaming_multTransposeImpl.cpp \
           $(DD)/operation/hash/OperationMultiEvalModMaskStreaming/OperationMultiEvalModMaskStreaming.cpp \
           $(DD)/operation/hash/OperationMultiEvalModMaskStreaming/OperationMultiEvalModMaskStreaming_multImpl.cpp \
           $(DD)/operation/hash/OperationMultiEvalModMaskStreaming/OperationMultiEvalModMaskStreaming_multTransposeImpl.cpp \
           $(DD)/tools/ARFFTools.cpp $(DD)/tools/CSVTools.cpp $(DD)/tools/Dataset.cpp \
           $(DD)/algorithm/SystemMatrixLeastSquaresIdentity.cpp \
           $(DD)/algorithm/DMSystemMatrixBase.cpp

REF_SRCS := $(BASE_SRCS) $(SOLVER_SRCS) $(DD_SRCS)
REF_OBJS := $(patsubst $(REF)/%.cpp,$(OBJ)/%.o,$(REF_SRCS))
HARNESS_OBJ := $(OBJ)/ref_harness.o

all: $(OUT)/libsgpp_ref.so

$(OBJ)/%.o: $(REF)/%.cpp
	@mkdir -p $(dir $@)
	$(CXX) $(CXXFLAGS) -c $< -o $@

$(HARNESS_OBJ): oracle/ref_harness.cpp
	@mkdir -p $(dir $@)
	$(CXX) $(CXXFLAGS) -c $< -o $@

$(OUT)/libsgpp_ref.so: $(REF_OBJS) $(HARNESS_OBJ)
	$(CXX) -shared -fopenmp -o $@ $^

.PHONY: all
