# Builds the reference's GPU miner (gspan_cuda_no_sort) for sm_103a, as a second
# oracle beside the sequential reference.  Test infrastructure only; outputs go
# to _ref/ (git-ignored, but carried to the GPU machine with the rest of the tree).
#
#   make -C oracle -f gspan_cuda.mk src REF=<reference tree>
#       copies the needed reference sources into _ref/gspan_cuda_src/ and applies
#       the patches CUDA 13 needs (run where the reference tree is present)
#   make -C oracle -f gspan_cuda.mk -j8
#       compiles _ref/gspan_cuda_src/ into _ref/gspan_cuda_ref (no reference tree
#       needed: the copied sources travel with _ref/)
#
# Patches (applied to the copy, never to the reference tree):
#   1. CCCL 3 dropped thrust::binary_function / unary_function: the functors'
#      base classes are removed (compute_support.cpp).
#   2. The extension record's copy and field constructors get __host__ __device__
#      (cuda_datastructures.hpp): Thrust/CUB 3 copy records in device code.
#   3. __ballot -> __ballot_sync(0xffffffff, ...) in the reduction library's
#      kernels, so that they compile; they are no longer called (4).
#   4. The reduction library's class bodies (cuda_segmented_scan,
#      cuda_segmented_reduction, cuda_copy) are replaced by Thrust versions
#      (gspan_cuda/reduction.cu, gspan_cuda/cuda_copy.tcc): its MGPU-era kernels
#      assume implicit warp lock-step, which GPUs since Volta do not give.
#      cucpp.cpp / mgpuscan.cpp (driver-API context code, unused) are left out.
REF ?= $(abspath $(CURDIR)/../../reference)
SRC := _ref/gspan_cuda_src
OBJ := _ref/gspan_cuda_obj
BIN := _ref/gspan_cuda_ref
NVCC ?= nvcc

GLOBALS := cuda_graph_types dbio dfs_code dfs_ismin graph_getmin graph_output graph_types logger utils \
           embedding_lists memory_checker
CUDAPP := cuda_configurator
GSPANCUDA := gspan_cuda gspan_cuda_no_sort compute_extensions compute_support first_embedding cuda_utils \
             filter_backward filter_rmpath gspan_cuda_tests
# gspan_cuda.cpp links its debugging checks (gspan_cuda_tests.cpp; two more from the
# gtest-based tests/test_embeddings.cpp, stood in for by gspan_cuda/test_stubs.cpp)
OBJS := $(addprefix $(OBJ)/g_,$(addsuffix .o,$(GLOBALS))) $(addprefix $(OBJ)/p_,$(addsuffix .o,$(CUDAPP))) \
        $(addprefix $(OBJ)/c_,$(addsuffix .o,$(GSPANCUDA))) $(OBJ)/test_stubs.o $(OBJ)/reduction.o \
        $(OBJ)/harness.o
FLAGS := -std=c++17 -O2 -w -DLOG_INFO -DSTLPORT_UNAVAL -gencode arch=compute_103a,code=sm_103a \
         -I$(SRC)/gspan_cuda -I$(SRC)/globals -I$(SRC)/cuda_pp -I$(SRC)/reduction -I$(SRC)/gspan

all: $(BIN)

src:
	rm -rf $(SRC)
	mkdir -p $(SRC)
	cp -r $(REF)/src/globals $(REF)/src/cuda_pp $(REF)/src/gspan_cuda $(REF)/src/reduction $(REF)/src/gspan $(SRC)/
	sed -i -e 's/: *public thrust::binary_function<[^>]*>//' -e 's/: *public thrust::unary_function<[^>]*>//' \
	    $(SRC)/gspan_cuda/*.cpp $(SRC)/gspan_cuda/*.hpp
	sed -i -e 's/^\( *\)extension_element_t(\(const extension_element_t\|int from\)/\1__host__ __device__ extension_element_t(\2/' \
	    $(SRC)/gspan_cuda/cuda_datastructures.hpp
	sed -i 's/__ballot(/__ballot_sync(0xffffffffu, /g' $(SRC)/reduction/*.cu
	cp gspan_cuda/cuda_copy.tcc $(SRC)/reduction/cuda_copy.tcc

$(OBJ)/g_%.o: $(SRC)/globals/%.cpp
	@mkdir -p $(OBJ)
	$(NVCC) -x cu $(FLAGS) -c $< -o $@
$(OBJ)/p_%.o: $(SRC)/cuda_pp/%.cpp
	@mkdir -p $(OBJ)
	$(NVCC) -x cu $(FLAGS) -c $< -o $@
$(OBJ)/c_%.o: $(SRC)/gspan_cuda/%.cpp
	@mkdir -p $(OBJ)
	$(NVCC) -x cu $(FLAGS) -c $< -o $@
$(OBJ)/test_stubs.o: gspan_cuda/test_stubs.cpp
	@mkdir -p $(OBJ)
	$(NVCC) -x cu $(FLAGS) -c $< -o $@
$(OBJ)/reduction.o: gspan_cuda/reduction.cu
	@mkdir -p $(OBJ)
	$(NVCC) $(FLAGS) -c $< -o $@
$(OBJ)/harness.o: gspan_cuda/harness.cpp
	@mkdir -p $(OBJ)
	$(NVCC) -x cu $(FLAGS) -c $< -o $@

$(BIN): $(OBJS)
	$(NVCC) -gencode arch=compute_103a,code=sm_103a -o $@ $(OBJS)

clean:
	rm -rf $(SRC) $(OBJ) $(BIN)

.PHONY: all src clean
