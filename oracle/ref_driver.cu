// ref_driver.cu -- a cross-check library built from the reference's own
// BLAZE_gpu sources, where they lie (the recipe in oracle/Makefile, target
// `ref`, compiles BLAZE_gpu/gpuBLAZE.cu, which includes util.hpp, with the
// stub NCBI and boost headers of oracle/ref_stubs). Test infrastructure only:
// it generates golden vectors from the reference's code to pin the oracle;
// the product never loads it, and no source of the reference is copied here.
//
// Exported:
//   ref_neighbouring_words  the reference's neighbourhood of one 3-letter word
//                           (BLAZE_gpu/util.hpp:64-85: every other word
//                           scoring >= 11 under its BLOSUM62 copy
//                           util.hpp:30-57; the word itself excluded)
//   ref_score               its BLOSUM62 copy, entry (a, b)
#include "gpuBLAZE.cu"

extern "C" int ref_neighbouring_words(int x, int y, int z, int *out, int cap) {
    if (x < 0 || y < 0 || z < 0 || x >= 28 || y >= 28 || z >= 28) return -1;
    const std::vector<int> v = neighbouring_words(x, y, z);
    const int n = static_cast<int>(v.size());
    for (int i = 0; i < n && i < cap; ++i) out[i] = v[i];
    return n;
}

extern "C" int ref_score(int a, int b) {
    if (a < 0 || b < 0 || a >= 28 || b >= 28) return 0;
    return matrix[a][b];
}
