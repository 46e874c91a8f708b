// fiuncho_gpu: command-line front end of the GPU search, with the reference
// CLI's arguments and output format (app/main.cpp:26-169 of Fiuncho):
//
//   fiuncho_gpu -o ORDER [-n NOUTPUTS] [-d DEVICE] INPUT... OUTPUT
//
// INPUT is one .raw file or a .tped + .tfam pair; OUTPUT receives one line
// "i j ... val" per result (Result::str), best first.  -d replaces the
// reference's -t THREADS: the search runs on CUDA device DEVICE.
#include <fiuncho/GpuSearch.h>
#include <fiuncho/MPIEngine.h>

#include <cstdlib>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

static int usage(const char *argv0, const std::string &msg)
{
    std::cerr << msg << "\nusage: " << argv0 << " -o ORDER [-n NOUTPUTS] [-d DEVICE] INPUT... OUTPUT\n";
    return 1;
}

int main(int argc, char **argv)
{
    int order = 0, outputs = 10, device = 0;
    std::vector<std::string> files;
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        auto value = [&](int &dst) {
            if (i + 1 >= argc) return false;
            char *end = nullptr;
            const long v = std::strtol(argv[++i], &end, 10);
            if (*end != '\0') return false;
            dst = (int)v;
            return true;
        };
        if (a == "-o" || a == "--order") {
            if (!value(order)) return usage(argv[0], "invalid ORDER");
        } else if (a == "-n" || a == "--noutputs") {
            if (!value(outputs)) return usage(argv[0], "invalid NOUTPUTS");
        } else if (a == "-d" || a == "--device") {
            if (!value(device)) return usage(argv[0], "invalid DEVICE");
        } else {
            files.push_back(a);
        }
    }
    if (order < 2) return usage(argv[0], "order is equal or greater than 2");
    if (outputs < 1) return usage(argv[0], "noutputs is greater than 0");
    if (files.size() < 2) return usage(argv[0], "input and output files (output goes last)");
    const std::string output = files.back();
    files.pop_back();
    try {
        MPIEngine engine;
        auto results = engine.run<GpuSearch>(files, (unsigned)order, (unsigned)outputs, device);
        std::ofstream of(output);
        if (!of) throw std::runtime_error("Cannot write into \"" + output + "\"");
        for (const auto &r : results) of << r.str() << '\n';
    } catch (const std::runtime_error &e) {
        std::cerr << e.what() << std::endl;
        return 1;
    }
    return 0;
}
