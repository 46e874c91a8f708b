/**
 * @file Readers.hpp
 * @brief Genotype codes and the bit packer of the host-side C++ mirror.
 * Files are parsed by the library (fiu_read_genotypes, threaded, with the
 * reference's input rules of include/fiuncho/dataset/TPEDFile.hpp and
 * RAWFile.hpp); the packer here builds the reference layout on the host
 * (TPEDFile.hpp:176-269): per class, samples shifted in most-significant-bit
 * first; the last, partial word of a row is right-aligned; padding words are
 * zero.
 */
#ifndef FIUNCHO_READERS_HPP
#define FIUNCHO_READERS_HPP

#include <cstdint>
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

} // namespace fiuncho_io

#endif
