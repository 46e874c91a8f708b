/**
 * @file Search.h
 * @brief Search interface of the host-side C++ mirror (same declaration as the
 * reference's include/fiuncho/Search.h:19-46): one process's share of the
 * exhaustive search, described by a Distribution, returning its top results.
 */
#ifndef FIUNCHO_SEARCH_H
#define FIUNCHO_SEARCH_H

#include <fiuncho/Dataset.h>
#include <fiuncho/Distribution.h>
#include <fiuncho/utils/Result.h>

#include <cstdint>
#include <vector>

class Search
{
  public:
    virtual ~Search() {}

    virtual std::vector<Result<int, float>> run(const Dataset<uint64_t> &dataset, const unsigned short order,
                                                const Distribution<int> &distribution,
                                                const unsigned int outputs) = 0;
};

#endif
