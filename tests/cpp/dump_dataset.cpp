// Reads a data set with the C++ mirror's Dataset<uint64_t>::read and writes
// "snps cases ctrls cases_words ctrls_words" then the packed words (binary,
// native byte order) to OUT, for comparison with the reference's packing.
//   dump_dataset OUT INPUT [INPUT]
#include <fiuncho/Dataset.h>

#include <cstdio>
#include <iostream>

int main(int argc, char **argv)
{
    if (argc < 3) return 2;
    std::vector<std::string> in(argv + 2, argv + argc);
    try {
        const auto d = Dataset<uint64_t>::read(in);
        FILE *f = std::fopen(argv[1], "wb");
        if (!f) return 3;
        const unsigned long long hdr[5] = {d.snps, d.cases, d.ctrls, d[0].cases_words, d[0].ctrls_words};
        std::fwrite(hdr, sizeof hdr, 1, f);
        const size_t per = 3 * (d[0].cases_words + d[0].ctrls_words);
        std::fwrite(d[0].cases, sizeof(uint64_t), d.snps * per, f);
        std::fclose(f);
    } catch (const std::runtime_error &e) {
        std::cerr << e.what() << std::endl;
        return 1;
    }
    return 0;
}
