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

#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

template <class T> class Dataset
{
  public:
    Dataset(const Dataset<T> &) = delete;
    Dataset(Dataset<T> &&) = default;

    static Dataset<T> read(const std::vector<std::string> &inputs)
    {
        fiuncho_io::Genotypes g;
        if (inputs.size() == 1) {
            const std::string ext = fiuncho_io::extension(inputs[0]);
            if (ext != ".raw") throw std::runtime_error("Unrecognized input file extension " + ext);
            g = fiuncho_io::read_raw(inputs[0]);
        } else if (inputs.size() == 2) {
            const std::string e1 = fiuncho_io::extension(inputs[0]), e2 = fiuncho_io::extension(inputs[1]);
            if (e1 != ".tped" && e1 != ".tfam") throw std::runtime_error("Unrecognized input file extension " + e1);
            if (e1 == e2 || (e2 != ".tped" && e2 != ".tfam"))
                throw std::runtime_error("Expecting a tfam file after \"" + inputs[0] + "\", but found a " + e2);
            g = e1 == ".tped" ? fiuncho_io::read_tped(inputs[0], inputs[1]) : fiuncho_io::read_tped(inputs[1], inputs[0]);
        } else {
            throw std::runtime_error("Unrecognized number of input files to Dataset factory constructor");
        }
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
