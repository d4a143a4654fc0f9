// Prints the multi-index tables of tsem_gpu::Correspondence for orders 0..max_M in
// the layout of oracle/ref_correspondence.cpp (TSEMLib's own Correspondence<3>), so
// the two outputs can be compared byte for byte.  Host only: no GPU is touched.
#include <cstdio>
#include <cstdlib>

#include "tsem_gpu.hpp"

int main(int argc, char** argv) {
    const int max_M = argc > 1 ? std::atoi(argv[1]) : 12;
    for (int M = 0; M <= max_M; ++M) {
        tsem_gpu::Correspondence c(M);
        std::printf("M %d %d\n", M, c.n_index());
        for (int order = 0; order <= M; ++order)
            std::printf("range %d %d %d\n", order, c.n_index_begin(order), c.n_index_end(order));
        for (int i = 0; i < c.n_index(); ++i) {
            tsem_gpu::Multiindex a = c.number2index(i);
            std::printf("num %d %d %d %d %d\n", i, a.index[0], a.index[1], a.index[2], c.index2number(a));
        }
    }
    return 0;
}
