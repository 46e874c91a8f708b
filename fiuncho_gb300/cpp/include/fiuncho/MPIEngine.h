/**
 * @file MPIEngine.h
 * @brief Single-process engine of the host-side C++ mirror with the reference
 * MPIEngine::run<T>(inputs, order, outputs, args...) signature
 * (include/fiuncho/MPIEngine.h:108-182): read the data set, take
 * Distribution(snps, order - 1, size, rank) with one rank, run T, then sort by
 * value descending (ties: ascending combination) and truncate to `outputs`.
 * Ranks beyond one are outside this build: one process drives one GPU.
 */
#ifndef FIUNCHO_MPIENGINE_H
#define FIUNCHO_MPIENGINE_H

#include <fiuncho/Search.h>

#include <algorithm>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

class MPIEngine
{
  public:
    const int mpi_size = 1;
    const int mpi_rank = 0;

    template <typename T, typename... Args>
    std::vector<Result<int, float>> run(const std::vector<std::string> &inputs, const unsigned int order,
                                        const unsigned int outputs, Args &&...args)
    {
        const auto dataset = Dataset<uint64_t>::read(inputs);
        if (dataset.snps > (size_t)std::numeric_limits<int>::max()) {
            throw std::runtime_error("Input data limit exceeded: Dataset contains more than " +
                                     std::to_string(std::numeric_limits<int>::max()) + " SNPs");
        }
        const Distribution<int> distribution((int)dataset.snps, (int)order - 1, mpi_size, mpi_rank);
        std::unique_ptr<Search> search(new T(std::forward<Args>(args)...));
        auto results = search->run(dataset, (unsigned short)order, distribution, outputs);
        std::stable_sort(results.begin(), results.end(), [](const Result<int, float> &a, const Result<int, float> &b) {
            return a.val > b.val || (a.val == b.val && a.combination < b.combination);
        });
        if (results.size() > outputs) results.resize(outputs);
        return results;
    }
};

#endif
