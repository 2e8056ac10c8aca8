# Links the reference's gpu_test driver against libgmr.so instead of its own
# engine source: the driver (gpu-engine/gpu_engine_test.cu), the schedule
# builder (build_schedule.cpp) and the headers stay unchanged; only
# gpu_engine.cu of the reference's recipe (gpu-engine/Makefile:41-42) is
# replaced by the library, which exports the same two entry points.
#
#   make -f g-mm-repair_gb300/gpu_test.mk GMR_REFERENCE=/path/to/g-mm-repair [OUT=gpu_test]
#
# NVML is loaded by the library at run time, so -lnvidia-ml is not needed.
HERE := $(dir $(abspath $(lastword $(MAKEFILE_LIST))))
GMR ?= $(HERE)gmr
GMR_REFERENCE ?= /root/reference
REF ?= $(GMR_REFERENCE)/gpu-engine
NVCC ?= nvcc
CUDA_ARCH ?= sm_103a
OUT ?= gpu_test

$(OUT): $(REF)/gpu_engine_test.cu $(REF)/build_schedule.cpp $(GMR)/libgmr.so
	$(NVCC) -O3 -std=c++17 -arch=$(CUDA_ARCH) -Xcompiler -fopenmp -I$(REF) -o $@ \
	    $(REF)/gpu_engine_test.cu $(REF)/build_schedule.cpp -L$(GMR) -lgmr -Xlinker -rpath,$(GMR) -lgomp

.PHONY: $(OUT)
