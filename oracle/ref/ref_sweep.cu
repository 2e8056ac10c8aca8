// Harness around the reference driver gpu-engine/gpu_engine_test.cu, built by
// oracle/Makefile into oracle/_ref.  TEST INFRASTRUCTURE ONLY (golden-vector
// generation).  The driver source is included unchanged from the reference
// tree with its main() renamed on the command line, which makes its
// run_cpu_reference_layered<S> (gpu_engine_test.cu:49-104) callable here.
#include "gpu_engine_test.cu"

// The driver refers to the two engine entry points; this harness never calls
// them (it runs only the CPU sweep), so they are stubs.
extern "C" void run_gpu_right_multiply_layered(int, int, int, int, const LayeredRule*, const int*, const int*,
                                               const float*, int, const float*, const GPUSchedule&, float*, int) {
    std::abort();
}
extern "C" void run_gpu_right_multiply_batched(int, int, int, int, const LayeredRule*, const int*, const int*,
                                               const float*, int, const float*, const GPUSchedule&, float*, int,
                                               int) {
    std::abort();
}

// Sequential run of the reference CPU sweep (one OpenMP thread, so the float
// accumulation order is the reference's sequential order).
void ref_cpu_layered(int semiring, const BuiltSchedule& bs, int cols, const std::vector<float>& V,
                     const std::vector<float>& x, int rows, void* y) {
    int alpha = bs.alpha;
    std::vector<int> vi(alpha > 0 ? alpha - 1 : 0), ci(alpha > 0 ? alpha - 1 : 0);
    for (int q = 1; q < alpha; ++q) {  // gpu_engine_test.cu:373-380
        int t = bs.term_orig[q];
        vi[q - 1] = (t - 1) / cols;
        ci[q - 1] = (t - 1) % cols;
    }
#ifdef _OPENMP
    omp_set_num_threads(1);
#endif
    if (semiring == 0)
        run_cpu_reference_layered<PlusTimes>(rows, alpha, bs.max_depth, bs.layered_levels, bs.emit_by_level,
                                             bs.term_emit, vi.data(), ci.data(), V.data(), x.data(), (float*)y);
    else if (semiring == 1)
        run_cpu_reference_layered<Boolean>(rows, alpha, bs.max_depth, bs.layered_levels, bs.emit_by_level,
                                           bs.term_emit, vi.data(), ci.data(), V.data(), x.data(), (int*)y);
    else
        run_cpu_reference_layered<Tropical>(rows, alpha, bs.max_depth, bs.layered_levels, bs.emit_by_level,
                                            bs.term_emit, vi.data(), ci.data(), V.data(), x.data(), (int*)y);
}
