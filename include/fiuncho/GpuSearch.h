/**
 * @file GpuSearch.h
 * @brief Search implementation that runs the whole exhaustive search on one
 * CUDA GPU (GB300, sm_103a) through the C ABI of libfiuncho_gpu.so
 * (fiuncho_gpu.h).
 *
 * Drop-in for ThreadedSearch behind the Search interface
 * (include/fiuncho/Search.h:19-46 of the Fiuncho tree): same run() signature,
 * same result contract -- at most `outputs` Result<int,float> sorted by value
 * descending (ties ordered by ascending combination), combinations of `order`
 * ascending 0-based SNP indices, covering exactly the combinations whose
 * (order-1)-prefix the Distribution owns.  Usable wherever a Search type is:
 *
 *     MPIEngine engine;
 *     auto results = engine.run<GpuSearch>({tped, tfam}, order, outputs, device);
 *
 * Errors are reported as std::runtime_error, like the reference.  There is no
 * CPU fallback: without a usable GPU the constructor throws.
 *
 * Multi-GPU: MPIEngine gives rank r of N the strided prefix share
 * Distribution(snps, order-1, N, r) (MPIEngine.h:133-134).  The tensor-core
 * kernels serve such a share themselves at orders 2, 3 and 4 (one-hot data),
 * with the reference's per-rank list; other shares run on the CUDA-core
 * kernels.  With shard_ranks = true a rank share
 * runs as shard r of N of the whole search instead (fiu_search_shard: equal
 * ranges of the tensor-core work units, every order); the rank's own list
 * then differs from the strided share's, but MPIEngine's gathered result is
 * the same:
 *
 *     engine.run<GpuSearch>({tped, tfam}, order, outputs, local_rank, true);
 */
#ifndef FIUNCHO_GPUSEARCH_H
#define FIUNCHO_GPUSEARCH_H

#include <fiuncho/Search.h>
#include <fiuncho_gpu.h>

#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

class GpuSearch : public Search
{
    fiu_ctx *ctx = nullptr;
    bool shard_ranks = false;

  public:
    /**
     * @param device CUDA device ordinal used by this search object
     * @param shard_ranks run a rank share Distribution(snps, order-1, N, r) as
     * shard r of N of the whole search (see above)
     */
    explicit GpuSearch(int device = 0, bool shard_ranks = false) : shard_ranks(shard_ranks)
    {
        if (fiu_create(device, &ctx) != FIU_OK) {
            throw std::runtime_error("GpuSearch: cannot create a context on CUDA device " +
                                     std::to_string(device));
        }
    }

    GpuSearch(const GpuSearch &) = delete;
    GpuSearch &operator=(const GpuSearch &) = delete;

    ~GpuSearch() { fiu_destroy(ctx); }

    std::vector<Result<int, float>> run(const Dataset<uint64_t> &dataset, const unsigned short order,
                                        const Distribution<int> &distribution,
                                        const unsigned int outputs) override
    {
        std::vector<Result<int, float>> results;
        if (dataset.snps == 0) {
            return results;
        }
        const size_t cw = dataset[0].cases_words, tw = dataset[0].ctrls_words;
        const size_t per_snp = 3 * (cw + tw);
        // GenotypeTable::make_array places the tables back to back; copy them
        // together only if a data set was assembled some other way.
        const uint64_t *base = dataset[0].cases;
        std::vector<uint64_t> packed;
        for (size_t i = 0; i < dataset.snps; ++i) {
            if (dataset[(int)i].cases != base + i * per_snp || dataset[(int)i].ctrls != base + i * per_snp + 3 * cw) {
                packed.resize(dataset.snps * per_snp);
                for (size_t j = 0; j < dataset.snps; ++j) {
                    std::memcpy(packed.data() + j * per_snp, dataset[(int)j].cases, 3 * cw * sizeof(uint64_t));
                    std::memcpy(packed.data() + j * per_snp + 3 * cw, dataset[(int)j].ctrls,
                                3 * tw * sizeof(uint64_t));
                }
                base = packed.data();
                break;
            }
        }
        const fiu_dataset d{base, dataset.snps, dataset.cases, dataset.ctrls, cw, tw};
        const fiu_distribution dist{distribution.n, distribution.k, distribution.step, distribution.offset};
        std::vector<int32_t> comb((size_t)outputs * order);
        std::vector<float> vals(outputs);
        unsigned count = 0;
        const bool rank_share = shard_ranks && distribution.n == (int)dataset.snps && distribution.k == order - 1 &&
                                distribution.step >= 1 && distribution.offset >= 0 &&
                                distribution.offset < distribution.step;
        const int rc = rank_share ? fiu_search_shard(ctx, &d, order, (unsigned)distribution.offset,
                                                     (unsigned)distribution.step, outputs, comb.data(), vals.data(),
                                                     &count)
                                  : fiu_search(ctx, &d, order, &dist, outputs, comb.data(), vals.data(), &count);
        if (rc != FIU_OK) {
            throw std::runtime_error(std::string("GpuSearch::run: ") + fiu_last_error(ctx));
        }
        results.resize(count);
        for (unsigned i = 0; i < count; ++i) {
            results[i].combination.assign(comb.begin() + (size_t)i * order, comb.begin() + (size_t)(i + 1) * order);
            results[i].val = vals[i];
        }
        return results;
    }
};

#endif
