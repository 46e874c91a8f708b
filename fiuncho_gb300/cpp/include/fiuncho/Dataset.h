/**
 * @file Dataset.h
 * @brief Dataset<T> of the host-side C++ mirror: `snps` single-SNP
 * GenotypeTables over `cases` + `ctrls` individuals, read from one .raw file
 * or a .tped + .tfam pair (the reference's include/fiuncho/Dataset.h:26-152,
 * same dispatch rules and error messages).
 */
#ifndef FIUNCHO_DATASET_H
#define FIUNCHO_DATASET_H

#include <fiuncho/GenotypeTable.h>
#include <fiuncho/dataset/Readers.hpp>
#include <fiuncho_gpu.h>

#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

template <class T> class Dataset
{
  public:
    Dataset(const Dataset<T> &) = delete;
    Dataset(Dataset<T> &&) = default;

    /** Parses the inputs with the library's threaded reader (fiu_read_genotypes,
     * `threads` host threads, 0 = all cores) and packs them; errors throw
     * std::runtime_error with the reader's message, as the reference does. */
    static Dataset<T> read(const std::vector<std::string> &inputs, int threads = 0)
    {
        if (inputs.size() != 1 && inputs.size() != 2)
            throw std::runtime_error("Unrecognized number of input files to Dataset factory constructor");
        fiu_genotypes *h = nullptr;
        if (fiu_read_genotypes(nullptr, inputs[0].c_str(), inputs.size() == 2 ? inputs[1].c_str() : nullptr, threads,
                               &h) != FIU_OK)
            throw std::runtime_error(fiu_last_error(nullptr));
        uint64_t snps = 0, samples = 0;
        const uint8_t *codes = nullptr, *cases = nullptr;
        fiu_genotypes_info(h, &snps, &samples, &codes, &cases);
        fiuncho_io::Genotypes g;
        g.snps = snps;
        g.geno.assign(codes, codes + snps * samples);
        g.is_case.assign(cases, cases + samples);
        fiu_genotypes_free(h);
        return from_genotypes(g);
    }

    /** Packs minor-allele counts (g.geno[snp * samples + s] in {0,1,2}). */
    static Dataset<T> from_genotypes(const fiuncho_io::Genotypes &g, const size_t align = 0)
    {
        size_t cases = 0;
        for (auto c : g.is_case) cases += c ? 1 : 0;
        const size_t ctrls = g.is_case.size() - cases;
        const size_t cw = fiuncho_io::words_for(cases, align), tw = fiuncho_io::words_for(ctrls, align);
        auto arr = GenotypeTable<T>::make_array(g.snps, 1, cw, tw);
        for (size_t i = 0; i < g.snps; ++i)
            fiuncho_io::pack_snp(g.geno.data() + i * g.is_case.size(), g.is_case, cw, tw, arr[i].cases, arr[i].ctrls);
        return Dataset<T>(cases, ctrls, g.snps, arr);
    }

    GenotypeTable<T> &operator[](int i) { return data[i]; }
    const GenotypeTable<T> &operator[](int i) const { return data[i]; }

    const size_t cases;
    const size_t ctrls;
    const size_t snps;
    GenotypeTable<T> *data;

  private:
    Dataset(size_t c, size_t t, size_t s, std::unique_ptr<GenotypeTable<T>[]> &p)
        : cases(c), ctrls(t), snps(s), data(p.get()), array(std::move(p))
    {
    }

    std::unique_ptr<GenotypeTable<T>[]> array;
};

#endif
