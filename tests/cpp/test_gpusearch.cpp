// C++ parity test of the GpuSearch drop-in, written as the reference's own
// tests/threadedsearch.cpp and tests/mpiengine.cpp are (same checks): for
// orders 2..4, top-90 is non-empty, has 90 entries for order > 2, combinations
// of the right length, no repeats, strictly ascending indices; at order 3 the
// values normalised by the maximum match the MPI3SNP list within 5e-4.
//
//   test_gpusearch DATA.raw MPI3SNP.txt     (MPI3SNP.txt: "i j k value" lines)
#include <fiuncho/GpuSearch.h>
#include <fiuncho/MPIEngine.h>

#include <algorithm>
#include <cmath>
#include <fstream>
#include <iostream>
#include <map>
#include <set>
#include <sstream>
#include <string>
#include <vector>

static int failures = 0;
#define CHECK(cond, msg)                                                    \
    do {                                                                    \
        if (!(cond)) {                                                      \
            std::cerr << "FAIL: " << msg << " (" #cond ")" << std::endl;    \
            ++failures;                                                     \
        }                                                                   \
    } while (0)

static void common_checks(const std::vector<Result<int, float>> &r, int order, const std::string &what)
{
    CHECK(!r.empty(), what + ": empty result");
    if (order > 2) CHECK(r.size() == 90, what + ": 90 results");
    std::set<std::vector<int>> seen;
    for (const auto &x : r) {
        CHECK(x.combination.size() == (size_t)order, what + ": combination length");
        CHECK(seen.insert(x.combination).second, what + ": repeated combination");
        for (size_t i = 1; i < x.combination.size(); ++i)
            CHECK(x.combination[i - 1] < x.combination[i], what + ": ascending indices");
    }
    for (size_t i = 1; i < r.size(); ++i) CHECK(r[i - 1].val >= r[i].val, what + ": sorted");
}

static bool matches_mpi3snp(const std::vector<Result<int, float>> &r, const std::string &path)
{
    std::ifstream f(path);
    std::map<std::vector<int>, double> norm;
    std::string line;
    double first = 0;
    while (std::getline(f, line)) {
        std::istringstream s(line);
        std::vector<int> c(3);
        double v;
        if (!(s >> c[0] >> c[1] >> c[2] >> v)) continue;
        if (norm.empty()) first = v;
        norm[c] = v / first;
    }
    if (norm.empty() || r.empty()) return false;
    for (const auto &x : r) {
        auto it = norm.find(x.combination);
        const double want = it == norm.end() ? 0.0 : it->second;
        if (std::abs(x.val / r[0].val - want) > 0.0005) return false;
    }
    return true;
}

int main(int argc, char **argv)
{
    if (argc != 3) {
        std::cerr << "usage: test_gpusearch DATA.raw MPI3SNP.txt\n";
        return 2;
    }
    const auto dataset = Dataset<uint64_t>::read({argv[1]});
    CHECK(dataset.snps == 10 && dataset.cases == 9000 && dataset.ctrls == 9800, "data set shape");
    GpuSearch search(0);
    for (int o = 2; o < 5; ++o) {
        Distribution<int> distribution((int)dataset.snps, o - 1, 1, 0);
        auto r = search.run(dataset, o, distribution, 90);
        common_checks(r, o, "GpuSearch order " + std::to_string(o));
        if (o == 3) CHECK(matches_mpi3snp(r, argv[2]), "GpuSearch order 3 vs MPI3SNP");
    }
    MPIEngine engine;
    for (int o = 2; o < 5; ++o) {
        auto r = engine.run<GpuSearch>({argv[1]}, o, 90, 0);
        common_checks(r, o, "MPIEngine order " + std::to_string(o));
        if (o == 3) CHECK(matches_mpi3snp(r, argv[2]), "MPIEngine order 3 vs MPI3SNP");
    }
    // shard mode: the rank shares of 3 ranks run as shards of the whole search;
    // merged (value descending, combination ascending) they give the whole result
    GpuSearch sharded(0, true);
    for (int o = 2; o < 5; ++o) {
        Distribution<int> whole((int)dataset.snps, o - 1, 1, 0);
        auto ref = search.run(dataset, o, whole, 90);
        std::vector<Result<int, float>> merged;
        for (int r = 0; r < 3; ++r) {
            Distribution<int> share((int)dataset.snps, o - 1, 3, r);
            auto part = sharded.run(dataset, o, share, 90);
            merged.insert(merged.end(), part.begin(), part.end());
        }
        std::sort(merged.begin(), merged.end(), [](const Result<int, float> &a, const Result<int, float> &b) {
            return a.val != b.val ? a.val > b.val : a.combination < b.combination;
        });
        if (merged.size() > ref.size()) merged.resize(ref.size());
        std::map<std::vector<int>, float> want, got;
        for (const auto &x : ref) want[x.combination] = x.val;
        for (const auto &x : merged) got[x.combination] = x.val;
        CHECK(want == got, "sharded rank shares merge to the whole result, order " + std::to_string(o));
    }
    bool threw = false;
    try {
        Distribution<int> bad((int)dataset.snps, 1, 1, 0);
        search.run(dataset, 3, bad, 10);
    } catch (const std::runtime_error &) {
        threw = true;
    }
    CHECK(threw, "invalid distribution raises std::runtime_error");
    if (failures == 0) std::cout << "PASS" << std::endl;
    return failures ? 1 : 0;
}
