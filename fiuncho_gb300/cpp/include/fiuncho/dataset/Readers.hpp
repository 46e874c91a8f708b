/**
 * @file Readers.hpp
 * @brief PLINK .tped/.tfam and PLINK / GAMETES .raw readers and the bit
 * packer of the host-side C++ mirror.  Input rules follow the reference's
 * include/fiuncho/dataset/TPEDFile.hpp and RAWFile.hpp:
 *  - tfam phenotype (column 6): 1 = control, 2 = case, anything else an error;
 *  - tped nucleotides A/C/G/T, two per sample; the minor allele is the rarer
 *    of the two lexicographically smallest nucleotides (ties: the smaller);
 *  - raw: optional FID IID PAT MAT SEX prefix; phenotype column PHENOTYPE
 *    (1/2) or Class (GAMETES, 0/1); genotype columns are <id>_<A|C|G|T> or
 *    plain alphanumeric ids, other columns (e.g. *_HET) are skipped.
 * Packing: per class, samples shifted in most-significant-bit first; the last,
 * partial word of a row is right-aligned; padding words are zero.
 */
#ifndef FIUNCHO_READERS_HPP
#define FIUNCHO_READERS_HPP

#include <cstdint>
#include <fstream>
#include <regex>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace fiuncho_io
{

struct Genotypes {
    size_t snps = 0;
    std::vector<uint8_t> geno;   // snps x samples, minor-allele counts
    std::vector<bool> is_case;   // per sample
};

inline std::string extension(const std::string &path)
{
    const auto slash = path.find_last_of('/');
    const auto dot = path.find_last_of('.');
    if (dot == std::string::npos || (slash != std::string::npos && dot < slash)) return "";
    return path.substr(dot);
}

inline size_t words_for(size_t n, size_t align)
{
    if (align) return (n + align * 8 - 1) / (align * 8) * (align / 8);
    return (n + 63) / 64;
}

template <typename T>
void pack_snp(const uint8_t *g, const std::vector<bool> &is_case, size_t cw, size_t tw, T *cases, T *ctrls)
{
    constexpr size_t BITS = sizeof(T) * 8;
    T buf[2][3] = {{0, 0, 0}, {0, 0, 0}};
    size_t cnt[2] = {0, 0};
    T *dst[2] = {cases, ctrls};
    const size_t words[2] = {cw, tw};
    for (size_t k = 0; k < 3 * cw; ++k) cases[k] = 0;
    for (size_t k = 0; k < 3 * tw; ++k) ctrls[k] = 0;
    for (size_t s = 0; s < is_case.size(); ++s) {
        const int c = is_case[s] ? 0 : 1;
        for (int k = 0; k < 3; ++k) buf[c][k] = (T)((buf[c][k] << 1) | (T)(g[s] == k));
        if (++cnt[c] % BITS == 0) {
            for (int k = 0; k < 3; ++k) {
                dst[c][k * words[c] + cnt[c] / BITS - 1] = buf[c][k];
                buf[c][k] = 0;
            }
        }
    }
    for (int c = 0; c < 2; ++c)
        if (cnt[c] % BITS)
            for (int k = 0; k < 3; ++k) dst[c][k * words[c] + cnt[c] / BITS] = buf[c][k];
}

inline std::vector<std::string> split(const std::string &line)
{
    std::istringstream s(line);
    std::vector<std::string> out;
    std::string w;
    while (s >> w) out.push_back(w);
    return out;
}

inline Genotypes read_tped(const std::string &tped, const std::string &tfam)
{
    Genotypes g;
    std::ifstream fam(tfam);
    if (!fam) throw std::runtime_error("Error while opening " + tfam + ", check file path/permissions");
    std::string line;
    size_t ln = 0;
    while (std::getline(fam, line)) {
        ++ln;
        auto t = split(line);
        if (t.empty()) continue;
        if (t.size() < 6 || (t[5] != "1" && t[5] != "2"))
            throw std::runtime_error("Error in " + tfam + ":" + std::to_string(ln) + ": parsing error");
        g.is_case.push_back(t[5] == "2");
    }
    const size_t n = g.is_case.size();
    std::ifstream ped(tped);
    if (!ped) throw std::runtime_error("Error while opening " + tped + ", check file path/permissions");
    ln = 0;
    while (std::getline(ped, line)) {
        ++ln;
        auto t = split(line);
        if (t.empty()) continue;
        const std::string where = "Error in " + tped + ":" + std::to_string(ln) + ": ";
        if (t.size() < 4) throw std::runtime_error(where + "invalid loci information");
        std::string al;
        for (size_t i = 4; i < t.size(); ++i) al += t[i];
        size_t cnt[4] = {0, 0, 0, 0};
        const std::string acgt = "ACGT";
        for (char c : al) {
            const auto p = acgt.find(c);
            if (p == std::string::npos) throw std::runtime_error(where + "invalid nucleotide value '" + c + "'");
            ++cnt[p];
        }
        if (al.size() % 2) throw std::runtime_error(where + "odd number of nucleotides");
        if (al.size() != 2 * n)
            throw std::runtime_error(where + "the number of nucleotides does not match the number of samples");
        int a1 = -1, a2 = -1;
        for (int i = 0; i < 4; ++i)
            if (cnt[i]) {
                if (a1 < 0) a1 = i;
                else if (a2 < 0) a2 = i;
            }
        const char minor = a2 < 0 ? 0 : acgt[cnt[a1] > cnt[a2] ? a2 : a1];
        for (size_t s = 0; s < n; ++s) g.geno.push_back((uint8_t)((al[2 * s] == minor) + (al[2 * s + 1] == minor)));
        ++g.snps;
    }
    return g;
}

inline Genotypes read_raw(const std::string &path)
{
    std::ifstream f(path);
    if (!f) throw std::runtime_error("Error while opening " + path + ", check file path/permissions");
    std::string header;
    std::getline(f, header);
    std::vector<std::string> words;
    const std::regex word("(\\w+)");
    for (auto it = std::sregex_iterator(header.begin(), header.end(), word); it != std::sregex_iterator(); ++it)
        words.push_back(it->str());
    size_t info = 0;
    const char *names[5] = {"FID", "IID", "PAT", "MAT", "SEX"};
    while (info < 5 && info < words.size() && words[info] == names[info]) ++info;
    const bool has_info = info == 5;
    const std::vector<std::string> cols(words.begin() + (has_info ? 5 : 0), words.end());
    const std::regex geno_col("(\\w+_[ACGT])|([[:alnum:]]+)");
    long ph = -1;
    std::vector<bool> keep(cols.size());
    for (size_t i = 0; i < cols.size(); ++i) {
        if (cols[i] == "PHENOTYPE" || cols[i] == "Class") {
            if (ph >= 0) throw std::runtime_error("Error while parsing \"" + path + "\", multiple phenotype columns found");
            ph = (long)i;
        } else {
            keep[i] = std::regex_match(cols[i], geno_col);
        }
    }
    if (ph < 0) throw std::runtime_error("Error while parsing \"" + path + "\", no phenotype column");
    std::vector<std::vector<uint8_t>> per_sample;
    Genotypes g;
    std::string line;
    while (std::getline(f, line)) {
        auto t = split(line);
        if (t.empty()) continue;
        if (t.size() != cols.size() + (has_info ? 5 : 0))
            throw std::runtime_error("Error while parsing \"" + path + "\": ragged row");
        std::vector<uint8_t> v;
        for (size_t i = 0; i < cols.size(); ++i) {
            const std::string &x = t[i + (has_info ? 5 : 0)];
            size_t pos = 0;
            long val = 0;
            try {
                val = std::stol(x, &pos);
            } catch (const std::exception &) {
                pos = 0;
            }
            if (pos != x.size()) throw std::runtime_error("Error while parsing \"" + path + "\": non-numeric field");
            if ((long)i == ph) g.is_case.push_back(val + (has_info ? 0 : 1) != 1);
            else if (keep[i]) v.push_back((uint8_t)val);
        }
        per_sample.push_back(std::move(v));
    }
    g.snps = per_sample.empty() ? 0 : per_sample[0].size();
    const size_t n = per_sample.size();
    g.geno.resize(g.snps * n);
    for (size_t s = 0; s < n; ++s)
        for (size_t i = 0; i < g.snps; ++i) g.geno[i * n + s] = per_sample[s][i];
    return g;
}

} // namespace fiuncho_io

#endif
