/*
 * ref_driver.cpp -- C entry points over the UNMODIFIED reference sources
 * (headers under include/fiuncho/ and one src/<isa>/ kernel set), compiled by
 * oracle/ref/build_ref.sh into oracle/_ref/.  TEST INFRASTRUCTURE ONLY: used in
 * the development container to pin the oracle restatement and to produce the
 * golden fixtures under tests/golden/.  Never shipped, never the product.
 *
 * Everything below calls the reference's own public API:
 *   Dataset<uint64_t>::read          (include/fiuncho/Dataset.h:48-94)
 *   ThreadedSearch::run              (include/fiuncho/ThreadedSearch.h:207-246)
 *   MPIEngine::run<ThreadedSearch>   (include/fiuncho/MPIEngine.h:108-182), 1 rank
 *   GenotypeTable::combine / combine_and_popcnt (GenotypeTable.h:123-140)
 *   MutualInformation<float>::compute (MutualInformation.h:58-84)
 * The only non-public step is building a Dataset from an already packed
 * buffer (the Dataset constructor is private, Dataset.h:144-149); it is
 * reached by widening access for that one header include below.
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
#include <regex>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "mpi.h"
#include "tabledigest.h"

#define private public
#include <fiuncho/Dataset.h>
#undef private
#include <fiuncho/ContingencyTable.h>
#include <fiuncho/Distribution.h>
#include <fiuncho/GenotypeTable.h>
#include <fiuncho/MPIEngine.h>
#include <fiuncho/ThreadedSearch.h>
#include <fiuncho/algorithms/MutualInformation.h>

namespace {
thread_local std::string g_err;

struct Handle {
    std::unique_ptr<Dataset<uint64_t>> d;
};

Handle *wrap(Dataset<uint64_t> &&d)
{
    auto h = new Handle;
    h->d.reset(new Dataset<uint64_t>(std::move(d)));
    return h;
}

long copy_results(const std::vector<Result<int, float>> &r, int order, int32_t *combos, float *vals, long cap)
{
    long n = std::min<long>((long)r.size(), cap);
    for (long i = 0; i < n; ++i) {
        for (int j = 0; j < order; ++j) combos[i * order + j] = r[i].combination[j];
        vals[i] = r[i].val;
    }
    return n;
}
} // namespace

extern "C" {

const char *ref_last_error() { return g_err.c_str(); }

int ref_align() {
#ifdef ALIGN
    return ALIGN;
#else
    return 0;
#endif
}

/* Load one .raw or a .tped + .tfam pair with Dataset<uint64_t>::read. */
void *ref_read(const char *f1, const char *f2)
{
    try {
        std::vector<std::string> in{f1};
        if (f2 && *f2) in.emplace_back(f2);
        return wrap(Dataset<uint64_t>::read(in));
    } catch (const std::exception &e) {
        g_err = e.what();
        return nullptr;
    }
}

/* Build a Dataset from a buffer packed in the reference layout. */
void *ref_from_packed(const uint64_t *data, size_t snps, size_t cases, size_t ctrls, size_t cw, size_t tw)
{
    auto arr = GenotypeTable<uint64_t>::make_array(snps, 1, cw, tw);
    for (size_t i = 0; i < snps; ++i) {
        std::memcpy(arr[i].cases, data + i * 3 * (cw + tw), 3 * cw * sizeof(uint64_t));
        std::memcpy(arr[i].ctrls, data + i * 3 * (cw + tw) + 3 * cw, 3 * tw * sizeof(uint64_t));
    }
    return wrap(Dataset<uint64_t>(cases, ctrls, snps, arr));
}

void ref_free(void *h) { delete (Handle *)h; }

void ref_info(void *h, size_t *out /* snps, cases, ctrls, cases_words, ctrls_words */)
{
    const auto &d = *((Handle *)h)->d;
    out[0] = d.snps;
    out[1] = d.cases;
    out[2] = d.ctrls;
    out[3] = d[0].cases_words;
    out[4] = d[0].ctrls_words;
}

/* Copy the packed data out in the reference layout (3 case rows, 3 ctrl rows per SNP). */
void ref_packed(void *h, uint64_t *out)
{
    const auto &d = *((Handle *)h)->d;
    const size_t cw = d[0].cases_words, tw = d[0].ctrls_words;
    for (size_t i = 0; i < d.snps; ++i) {
        std::memcpy(out + i * 3 * (cw + tw), d[i].cases, 3 * cw * sizeof(uint64_t));
        std::memcpy(out + i * 3 * (cw + tw) + 3 * cw, d[i].ctrls, 3 * tw * sizeof(uint64_t));
    }
}

/* ThreadedSearch(threads).run(dataset, order, Distribution(n, order-1, step, offset), outputs). */
long ref_search(void *h, int order, int threads, int step, int offset, unsigned outputs, int32_t *combos,
                float *vals)
{
    try {
        const auto &d = *((Handle *)h)->d;
        ThreadedSearch s(threads);
        Distribution<int> dist((int)d.snps, order - 1, step, offset);
        auto r = s.run(d, order, dist, outputs);
        return copy_results(r, order, combos, vals, outputs);
    } catch (const std::exception &e) {
        g_err = e.what();
        return -1;
    }
}

/* MPIEngine().run<ThreadedSearch>(inputs, order, outputs, threads) at one rank. */
long ref_engine(const char *f1, const char *f2, int order, int threads, unsigned outputs, int32_t *combos,
                float *vals)
{
    try {
        std::vector<std::string> in{f1};
        if (f2 && *f2) in.emplace_back(f2);
        MPIEngine engine;
        auto r = engine.run<ThreadedSearch>(in, order, outputs, threads);
        return copy_results(r, order, combos, vals, outputs);
    } catch (const std::exception &e) {
        g_err = e.what();
        return -1;
    }
}

/* Contingency tables (3^order cells per class, padding dropped) of the given
 * combinations via chained combine + combine_and_popcnt, and their reference
 * FP32 MI. */
int ref_tables(void *h, int order, const int32_t *combos, size_t count, uint32_t *cases_out, uint32_t *ctrls_out,
               float *mi_out)
{
    const auto &d = *((Handle *)h)->d;
    const size_t cw = d[0].cases_words, tw = d[0].ctrls_words;
    size_t cells = 1;
    for (int i = 0; i < order; ++i) cells *= 3;
    std::vector<GenotypeTable<uint64_t>> gts;
    gts.reserve(order);
    for (int o = 2; o < order; ++o) gts.emplace_back(o, cw, tw);
    ContingencyTable<uint32_t> ct(order);
    MutualInformation<float> mi(d.cases, d.ctrls);
    for (size_t q = 0; q < count; ++q) {
        const int32_t *c = combos + q * order;
        for (int i = 0; i < order - 2; ++i)
            GenotypeTable<uint64_t>::combine(i > 0 ? gts[i - 1] : d[c[0]], d[c[i + 1]], gts[i]);
        GenotypeTable<uint64_t>::combine_and_popcnt(order > 2 ? gts.back() : d[c[0]], d[c[order - 1]], ct);
        std::memcpy(cases_out + q * cells, ct.cases, cells * sizeof(uint32_t));
        std::memcpy(ctrls_out + q * cells, ct.ctrls, cells * sizeof(uint32_t));
        if (mi_out) mi_out[q] = mi.compute(ct);
    }
    return 0;
}

/* MutualInformation<float>(n_cases, n_ctrls).compute over given tables of 3^order cells. */
int ref_mi(int order, const uint32_t *cases, const uint32_t *ctrls, size_t count, unsigned n_cases,
           unsigned n_ctrls, float *out)
{
    size_t cells = 1;
    for (int i = 0; i < order; ++i) cells *= 3;
    ContingencyTable<uint32_t> ct(order);
    for (size_t i = 0; i < ct.size; ++i) ct.cases[i] = ct.ctrls[i] = 0;
    MutualInformation<float> mi(n_cases, n_ctrls);
    for (size_t q = 0; q < count; ++q) {
        std::memcpy(ct.cases, cases + q * cells, cells * sizeof(uint32_t));
        std::memcpy(ct.ctrls, ctrls + q * cells, cells * sizeof(uint32_t));
        out[q] = mi.compute(ct);
    }
    return 0;
}

/* Digest (tabledigest.h) of the contingency tables of every combination a
 * Distribution(snps, order-1, step, offset) owns, visited exactly as
 * ThreadedSearch::nonsegmented_search visits them (ThreadedSearch.h:142-182):
 * each of `threads` threads owns distribution.layer(threads, t), builds the
 * prefix table with chained GenotypeTable::combine and fills each table with
 * GenotypeTable::combine_and_popcnt.  *count receives the combinations hashed. */
int ref_table_digest(void *h, int order, int threads, int step, int offset, uint64_t *digest, uint64_t *count)
{
    try {
        const auto &d = *((Handle *)h)->d;
        const Distribution<int> dist((int)d.snps, order - 1, step, offset);
        int cells = 1;
        for (int i = 0; i < order; ++i) cells *= 3;
        std::vector<uint64_t> sums(threads, 0), counts(threads, 0);
        std::vector<std::thread> ts;
        for (int t = 0; t < threads; ++t)
            ts.emplace_back([&, t]() {
                std::vector<GenotypeTable<uint64_t>> gts;
                gts.reserve(order);
                for (int o = 2; o < order; ++o) gts.emplace_back(o, d[0].cases_words, d[0].ctrls_words);
                ContingencyTable<uint32_t> ct(order);
                std::vector<int> comb(order);
                const Distribution<int> mine = dist.layer(threads, t);
                uint64_t s = 0, cnt = 0;
                for (auto c = mine.begin(); c < mine.end(); ++c) {
                    for (int i = 0; i < order - 2; ++i)
                        GenotypeTable<uint64_t>::combine(i > 0 ? gts[i - 1] : d[c[0]], d[c[i + 1]], gts[i]);
                    for (int i = 0; i < order - 1; ++i) comb[i] = c[i];
                    for (int l = c->back() + 1; l < (int)d.snps; ++l) {
                        GenotypeTable<uint64_t>::combine_and_popcnt(order > 2 ? gts.back() : d[c[0]], d[l], ct);
                        comb[order - 1] = l;
                        s += td_term(comb.data(), order, d.snps, ct.cases, ct.ctrls, cells);
                        ++cnt;
                    }
                }
                sums[t] = s;
                counts[t] = cnt;
            });
        uint64_t s = 0, cnt = 0;
        for (int t = 0; t < threads; ++t) {
            ts[t].join();
            s += sums[t];
            cnt += counts[t];
        }
        *digest = s;
        *count = cnt;
        return 0;
    } catch (const std::exception &e) {
        g_err = e.what();
        return -1;
    }
}

} // extern "C"

