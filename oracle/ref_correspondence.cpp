// TEST INFRASTRUCTURE ONLY: a driver around TSEMLib's own multi-index code.
//
// include/Correspondence.h and include/Multiindex.h (the lexicographic number <->
// multi-index maps of include/Correspondence.h:64-109) need nothing beyond the C++
// standard library, so this file compiles them where they lie in the reference tree
// (the Makefile's `ref` target passes their directory with -I) and prints, for each
// truncation order M = 0..max_M, every map the rest of TSEMLib reads from a
// Correspondence<3>:
//   M <M> <n_index()>
//   range <order> <n_index_begin(order)> <n_index_end(order)>     order = 0..M
//   num <i> <a0> <a1> <a2> <index2number(number2index(i))>         i = 0..n_index()-1
// The output is the golden fixture that pins the oracle's and the library's
// multi-index numbering to the reference's own code.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "Correspondence.h"

int main(int argc, char** argv) {
    const int max_M = argc > 1 ? std::atoi(argv[1]) : 12;
    if (max_M < 0 || max_M > 40) {
        std::fprintf(stderr, "max order out of range\n");
        return 2;
    }
    for (int M = 0; M <= max_M; ++M) {
        Correspondence<3> c(M);
        std::printf("M %d %d\n", M, c.n_index());
        for (int order = 0; order <= M; ++order)
            std::printf("range %d %d %d\n", order, c.n_index_begin(order), c.n_index_end(order));
        for (int i = 0; i < c.n_index(); ++i) {
            Multiindex<3> a = c.number2index(i);
            std::printf("num %d %d %d %d %d\n", i, a.index[0], a.index[1], a.index[2], c.index2number(a));
        }
    }
    return 0;
}
