// ref_tool: runs the reference's own CPU code on a grammar and writes its
// outputs, for the golden fixtures in tests/golden.  TEST INFRASTRUCTURE ONLY.
//
//   ref_tool <base> <rows> <cols> <x_prefix> <out_prefix>
//
// Reads <base>.vc.R/.vc.C/.val (format of gpu_engine_test.cu:291-345) and, for
// each semiring s in {plustimes, boolean, tropical}, <x_prefix>.<s>.x (cols
// float32).  Writes, from the reference's code:
//   <out_prefix>.<s>.y64  FP64 cpu_sweep               (cpu_selftest.cpp:67-102)
//   <out_prefix>.<s>.ybf  FP64 brute force on CSRV      (cpu_selftest.cpp:105-117)
//   <out_prefix>.<s>.y32  float/int sequential CPU sweep (gpu_engine_test.cu:49-104)
//   <out_prefix>.sched    int64 header + the flattened BuiltSchedule arrays
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

#include "build_schedule.h"
#include "grammar.h"

void ref_cpu_layered(int semiring, const BuiltSchedule& bs, int cols, const std::vector<float>& V,
                     const std::vector<float>& x, int rows, void* y);
std::vector<double> ref_sweep_f64(int semiring, const BuiltSchedule& bs, const std::vector<double>& V,
                                  const std::vector<float>& x, int rows, int cols);
std::vector<double> ref_brute(int semiring, const grammar::Grammar& g, const std::vector<double>& V,
                              const std::vector<float>& x, int rows, int cols);

template <class T>
static std::vector<T> slurp(const std::string& p) {
    std::ifstream f(p, std::ios::binary);
    if (!f) { std::fprintf(stderr, "cannot open %s\n", p.c_str()); std::exit(2); }
    f.seekg(0, std::ios::end);
    size_t n = (size_t)f.tellg() / sizeof(T);
    f.seekg(0);
    std::vector<T> v(n);
    f.read(reinterpret_cast<char*>(v.data()), (std::streamsize)(n * sizeof(T)));
    return v;
}
template <class T>
static void dump(std::ofstream& f, const std::vector<T>& v) {
    f.write(reinterpret_cast<const char*>(v.data()), (std::streamsize)(v.size() * sizeof(T)));
}

int main(int argc, char** argv) {
    if (argc != 6) { std::fprintf(stderr, "usage: ref_tool base rows cols x_prefix out_prefix\n"); return 1; }
    std::string base = argv[1], xp = argv[4], op = argv[5];
    int rows = std::stoi(argv[2]), cols = std::stoi(argv[3]);
    auto R = slurp<int>(base + ".vc.R");
    grammar::Grammar g;
    g.alpha = R[0];
    size_t nt = (R.size() - 1) / 2;
    g.rules.resize(nt);
    for (size_t i = 0; i < nt; ++i) g.rules[i] = {grammar::BINARY, R[1 + 2 * i], R[2 + 2 * i], 1};
    g.C = slurp<int>(base + ".vc.C");
    auto Vd = slurp<double>(base + ".val");
    std::vector<float> Vf(Vd.begin(), Vd.end());
    BuiltSchedule bs = build_schedule(g, rows, cols);
    const char* names[3] = {"plustimes", "boolean", "tropical"};
    for (int s = 0; s < 3; ++s) {
        auto x = slurp<float>(xp + "." + names[s] + ".x");
        if ((int)x.size() != cols) { std::fprintf(stderr, "x has %zu values, cols=%d\n", x.size(), cols); return 1; }
        auto y64 = ref_sweep_f64(s, bs, Vd, x, rows, cols);
        auto ybf = ref_brute(s, g, Vd, x, rows, cols);
        std::vector<int32_t> y32(rows);
        ref_cpu_layered(s, bs, cols, Vf, x, rows, y32.data());
        std::ofstream a(op + "." + names[s] + ".y64", std::ios::binary); dump(a, y64);
        std::ofstream b(op + "." + names[s] + ".ybf", std::ios::binary); dump(b, ybf);
        std::ofstream c(op + "." + names[s] + ".y32", std::ios::binary); dump(c, y32);
    }
    std::ofstream f(op + ".sched", std::ios::binary);
    std::vector<int64_t> head = {bs.alpha, bs.max_depth, bs.max_width, (int64_t)bs.num_raw_nt,
                                 (int64_t)bs.num_layered, (int64_t)bs.num_passthrough,
                                 (int64_t)bs.emit_pos.size(), (int64_t)bs.term_emit_sym.size()};
    dump(f, head);
    std::vector<int32_t> left, right;
    std::vector<float> coeff;
    for (auto& r : bs.flattened_rules) { left.push_back(r.left); right.push_back(r.right); coeff.push_back(r.coeff); }
    dump(f, left); dump(f, right); dump(f, coeff);
    dump(f, bs.level_offsets); dump(f, bs.emit_offsets); dump(f, bs.emit_pos); dump(f, bs.emit_row);
    dump(f, bs.term_emit_sym); dump(f, bs.term_emit_row); dump(f, bs.term_orig);
    return 0;
}
