// Harness around the reference self-test gpu-engine/cpu_selftest.cpp, built by
// oracle/Makefile into oracle/_ref.  TEST INFRASTRUCTURE ONLY.  The source is
// included unchanged with its main() renamed on the command line, which makes
// its FP64 cpu_sweep (cpu_selftest.cpp:67-102), brute_force (:105-117) and
// reconstruct_csrv (:149-156) callable here.
#include "cpu_selftest.cpp"

std::vector<double> ref_sweep_f64(int semiring, const BuiltSchedule& bs, const std::vector<double>& V,
                                  const std::vector<float>& x, int rows, int cols) {
    if (semiring == 1) return cpu_sweep<SRBool>(bs, V, x, rows, cols);
    if (semiring == 2) return cpu_sweep<SRTrop>(bs, V, x, rows, cols);
    return cpu_sweep<SRPlus>(bs, V, x, rows, cols);
}

std::vector<double> ref_brute(int semiring, const grammar::Grammar& g, const std::vector<double>& V,
                              const std::vector<float>& x, int rows, int cols) {
    std::vector<int> vc = reconstruct_csrv(g);
    if (semiring == 1) return brute_force<SRBool>(vc, V, x, rows, cols);
    if (semiring == 2) return brute_force<SRTrop>(vc, V, x, rows, cols);
    return brute_force<SRPlus>(vc, V, x, rows, cols);
}
