/*
 * bench_driver.cpp -- C entry points over the reference's two sequential
 * benchmark programs (benchmarks/nonsegmented_sequential_search.cpp and
 * benchmarks/segmented_sequential_search.cpp), compiled UNMODIFIED from where
 * they lie by oracle/build.py into oracle/_ref/libref_bench.so.  TEST
 * INFRASTRUCTURE ONLY: pins the oracle's restatement of their depth-first
 * traversal (orc_search_dfs) in the development container and produces the
 * fixtures of tests/golden/make_golden_traversals.py.  Never shipped.
 *
 * Each program is included in a namespace of its own with its main()
 * renamed; only its stack_search(dataset, order, maxarray) is called here.
 * Building a Dataset from a packed buffer widens access to the private
 * constructor (Dataset.h:144-149), as oracle/ref/ref_driver.cpp does.
 */
#include <algorithm>
#include <bitset>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <iostream>
#include <map>
#include <memory>
#include <pthread.h>
#include <regex>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <time.h>
#include <vector>

#include "mpi.h"

#define private public
#include <fiuncho/Dataset.h>
#undef private
#include <fiuncho/ContingencyTable.h>
#include <fiuncho/GenotypeTable.h>
#include <fiuncho/algorithms/MutualInformation.h>
#include <fiuncho/utils/MaxArray.h>
#include <fiuncho/utils/Result.h>
#include <fiuncho/utils/StaticStack.h>

namespace bench_nonseg {
#define main fiuncho_benchmark_main
#include "nonsegmented_sequential_search.cpp"
#undef main
}  // namespace bench_nonseg

namespace bench_seg {
#define main fiuncho_benchmark_main
#include "segmented_sequential_search.cpp"
#undef main
}  // namespace bench_seg

extern "C" {

/* stack_search of the segmented (segmented != 0) or non-segmented program on
 * a data set packed in the reference layout; the MaxArray's content sorted by
 * descending value (ties in the order the MaxArray holds them). */
long ref_stack_search(const uint64_t *data, size_t snps, size_t cases, size_t ctrls, size_t cw, size_t tw,
                      int order, int segmented, unsigned outputs, int32_t *combos, float *vals)
{
    try {
        auto arr = GenotypeTable<uint64_t>::make_array(snps, 1, cw, tw);
        for (size_t i = 0; i < snps; ++i) {
            std::memcpy(arr[i].cases, data + i * 3 * (cw + tw), 3 * cw * sizeof(uint64_t));
            std::memcpy(arr[i].ctrls, data + i * 3 * (cw + tw) + 3 * cw, 3 * tw * sizeof(uint64_t));
        }
        const Dataset<uint64_t> d(cases, ctrls, snps, arr);
        MaxArray<Result<int, float>> m(outputs);
        if (segmented) bench_seg::stack_search(d, (unsigned short)order, m);
        else bench_nonseg::stack_search(d, (unsigned short)order, m);
        std::vector<Result<int, float>> r;
        for (size_t i = 0; i < m.size(); ++i) r.push_back(m[i]);
        std::stable_sort(r.begin(), r.end(),
                         [](const Result<int, float> &a, const Result<int, float> &b) { return a.val > b.val; });
        for (size_t i = 0; i < r.size(); ++i) {
            for (int j = 0; j < order; ++j) combos[i * order + j] = r[i].combination[j];
            vals[i] = r[i].val;
        }
        return (long)r.size();
    } catch (const std::exception &e) {
        std::cerr << e.what() << "\n";
        return -1;
    }
}

}  // extern "C"
