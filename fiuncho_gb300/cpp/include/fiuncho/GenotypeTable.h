/**
 * @file GenotypeTable.h
 * @brief GenotypeTable<T> of the host-side C++ mirror: 3^order rows of
 * bit-packed samples for the cases followed by 3^order rows for the controls
 * (the reference's include/fiuncho/GenotypeTable.h:36-206).  make_array lays N
 * tables back to back in one allocation, which is the layout the GPU library
 * consumes directly.  The table arithmetic (combine, combine_and_popcnt) runs
 * on the GPU through fiu_combine / fiu_combine_and_popcnt.
 */
#ifndef FIUNCHO_GENOTYPETABLE_H
#define FIUNCHO_GENOTYPETABLE_H

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <memory>

template <class T> class GenotypeTable
{
  public:
    GenotypeTable(const GenotypeTable<T> &) = delete;
    GenotypeTable(GenotypeTable<T> &&) = default;

    GenotypeTable() : order(0), size(0), cases_words(0), ctrls_words(0), cases(nullptr), ctrls(nullptr) {}

    GenotypeTable(const short order, const size_t cases_words, const size_t ctrls_words)
        : order(order), size(pow3(order)), cases_words(cases_words), ctrls_words(ctrls_words),
          alloc(new T[pow3(order) * (cases_words + ctrls_words)](), std::default_delete<T[]>()),
          cases(alloc.get()), ctrls(cases + size * cases_words)
    {
    }

    static std::unique_ptr<GenotypeTable<T>[]> make_array(const size_t N, const short order,
                                                          const size_t cases_words, const size_t ctrls_words)
    {
        const size_t sz = pow3(order), per = sz * (cases_words + ctrls_words);
        std::shared_ptr<T> block(new T[N * per + 1](), std::default_delete<T[]>());
        auto arr = std::make_unique<GenotypeTable<T>[]>(N);
        for (size_t i = 0; i < N; ++i) {
            new (arr.get() + i) GenotypeTable<T>(order, cases_words, ctrls_words, block, block.get() + i * per,
                                                 block.get() + i * per + sz * cases_words);
        }
        return arr;
    }

    const size_t order;
    const size_t size;
    const size_t cases_words;
    const size_t ctrls_words;

  private:
    static size_t pow3(short o)
    {
        size_t r = 1;
        while (o-- > 0) r *= 3;
        return r;
    }

    GenotypeTable(const short order, const size_t cases_words, const size_t ctrls_words, std::shared_ptr<T> alloc,
                  T *cases, T *ctrls)
        : order(order), size(pow3(order)), cases_words(cases_words), ctrls_words(ctrls_words), alloc(alloc),
          cases(cases), ctrls(ctrls)
    {
    }

    std::shared_ptr<T> alloc;

  public:
    T *cases;
    T *ctrls;
};

#endif
