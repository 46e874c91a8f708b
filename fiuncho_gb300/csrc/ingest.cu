// Data set ingest: multi-threaded TPED/TFAM and RAW parsing into genotype
// codes, and packing of the codes on the device into the reference layout.
//
// Input rules are the reference's (include/fiuncho/dataset/TPEDFile.hpp:72-296,
// RAWFile.hpp:18-313, Dataset.h:48-94):
//  - tfam phenotype (column 6): 1 = control, 2 = case, anything else an error;
//  - tped: nucleotides A/C/G/T, two per sample; the minor allele is the rarer
//    of the two lexicographically smallest nucleotides present (ties: the
//    smaller), and a sample's genotype is its number of minor alleles;
//  - raw: optional FID IID PAT MAT SEX prefix; phenotype column PHENOTYPE
//    (1/2) or Class (GAMETES, 0/1); genotype columns are <id>_<A|C|G|T> or
//    plain alphanumeric ids, other columns (e.g. *_HET) are skipped.
// Parsing: the file is read whole, its line starts are found by all threads
// (one byte range each), then each thread parses a range of lines; an error
// reports the first failing line of the file, as a sequential reader would.
//
// Packing (TPEDFile.hpp:176-269): per SNP and class, three rows of
// `words` uint64 (genotype 0, 1, 2); samples of the class are shifted in
// most-significant-bit first, so in a full word the class's sample 64 w + b
// is bit 63 - b; the last, partial word of a row is right-aligned (its last
// sample is bit 0); words past the samples are zero.  On the device one warp
// builds a row set: its 32 lanes read 32 consecutive samples of the class,
// and three ballots per half word give the words.
#include <algorithm>
#include <atomic>
#include <cstdio>
#include <mutex>
#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "ctx.h"

struct fiu_genotypes {
    uint64_t snps = 0, samples = 0;
    std::vector<uint8_t> codes;    // snps x samples, minor-allele counts 0..2
    std::vector<uint8_t> is_case;  // per sample, 1 = case
};

using namespace fiu;

namespace {

struct Text {
    std::vector<char> buf;
    std::vector<size_t> line_start;  // start of every line (with the end of the text appended)
};

bool read_file(const std::string& path, std::vector<char>& buf) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    std::fseek(f, 0, SEEK_END);
    const long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    buf.resize(n > 0 ? (size_t)n : 0);
    const size_t got = n > 0 ? std::fread(buf.data(), 1, buf.size(), f) : 0;
    std::fclose(f);
    return got == buf.size();
}

// Line starts, found in parallel over byte ranges.
void split_lines(Text& t, int threads) {
    const size_t n = t.buf.size();
    const size_t T = (size_t)std::max(1, threads);
    std::vector<std::vector<size_t>> part(T);
    std::vector<std::thread> th;
    for (size_t p = 0; p < T; ++p)
        th.emplace_back([&, p] {
            const size_t a = n * p / T, b = n * (p + 1) / T;
            for (size_t i = a; i < b; ++i)
                if (t.buf[i] == '\n') part[p].push_back(i + 1);
        });
    for (auto& x : th) x.join();
    t.line_start.assign(1, 0);
    for (auto& v : part)
        for (size_t x : v)
            if (x < n) t.line_start.push_back(x);
    t.line_start.push_back(n);
}

// Whitespace-separated tokens of a line (pointer, length).
void tokens(const char* p, const char* e, std::vector<std::pair<const char*, size_t>>& out) {
    out.clear();
    while (p < e) {
        while (p < e && (*p == ' ' || *p == '\t' || *p == '\r' || *p == '\n' || *p == '\v' || *p == '\f')) ++p;
        const char* s = p;
        while (p < e && !(*p == ' ' || *p == '\t' || *p == '\r' || *p == '\n' || *p == '\v' || *p == '\f')) ++p;
        if (p > s) out.push_back({s, (size_t)(p - s)});
    }
}

// First error of a parallel pass: the smallest line number wins.
struct FirstError {
    std::atomic<size_t> line{~(size_t)0};
    std::string msg;
    std::mutex mu;
    void set(size_t ln, const std::string& m) {
        std::lock_guard<std::mutex> g(mu);
        if (ln < line.load()) {
            line.store(ln);
            msg = m;
        }
    }
};

template <class F>
void parallel_lines(size_t lines, int threads, F f) {
    const size_t T = (size_t)std::max(1, std::min<int>(threads, (int)std::max<size_t>(1, lines)));
    std::vector<std::thread> th;
    for (size_t p = 0; p < T; ++p) th.emplace_back([&, p] { f(lines * p / T, lines * (p + 1) / T); });
    for (auto& x : th) x.join();
}

std::string ext_of(const std::string& path) {
    const auto slash = path.find_last_of('/');
    const auto dot = path.find_last_of('.');
    if (dot == std::string::npos || (slash != std::string::npos && dot < slash)) return "";
    return path.substr(dot);
}

int read_tped(fiu_ctx* ctx, const std::string& tped, const std::string& tfam, int threads, fiu_genotypes& g) {
    // tfam: small, sequential
    std::vector<char> fam;
    if (!read_file(tfam, fam)) return fail(ctx, FIU_ERR_INVALID, "Error while opening " + tfam + ", check file path/permissions");
    {
        std::vector<std::pair<const char*, size_t>> t;
        size_t ln = 0, a = 0;
        while (a < fam.size()) {
            size_t b = a;
            while (b < fam.size() && fam[b] != '\n') ++b;
            ++ln;
            tokens(fam.data() + a, fam.data() + b, t);
            if (!t.empty()) {
                const bool one = t.size() >= 6 && t[5].second == 1 && (t[5].first[0] == '1' || t[5].first[0] == '2');
                if (!one) return fail(ctx, FIU_ERR_INVALID, "Error in " + tfam + ":" + std::to_string(ln) + ": parsing error");
                g.is_case.push_back(t[5].first[0] == '2');
            }
            a = b + 1;
        }
    }
    const size_t n = g.is_case.size();
    g.samples = n;
    Text txt;
    if (!read_file(tped, txt.buf))
        return fail(ctx, FIU_ERR_INVALID, "Error while opening " + tped + ", check file path/permissions");
    split_lines(txt, threads);
    const size_t lines = txt.line_start.size() - 1;
    // pass 1: which lines hold a SNP (non-empty), giving each its SNP index
    std::vector<uint8_t> nonempty(lines, 0);
    parallel_lines(lines, threads, [&](size_t a, size_t b) {
        for (size_t l = a; l < b; ++l)
            for (size_t i = txt.line_start[l]; i < txt.line_start[l + 1]; ++i) {
                const char c = txt.buf[i];
                if (!(c == ' ' || c == '\t' || c == '\r' || c == '\n' || c == '\v' || c == '\f')) {
                    nonempty[l] = 1;
                    break;
                }
            }
    });
    std::vector<size_t> snp_of(lines);
    size_t snps = 0;
    for (size_t l = 0; l < lines; ++l) {
        snp_of[l] = snps;
        snps += nonempty[l];
    }
    g.snps = snps;
    try {
        g.codes.assign(snps * n, 0);
    } catch (const std::exception&) {
        return fail(ctx, FIU_ERR_NOMEM, "genotype codes");
    }
    FirstError err;
    parallel_lines(lines, threads, [&](size_t a, size_t b) {
        std::vector<std::pair<const char*, size_t>> t;
        std::vector<uint8_t> al;
        for (size_t l = a; l < b; ++l) {
            if (!nonempty[l]) continue;
            if (l >= err.line) return;
            tokens(txt.buf.data() + txt.line_start[l], txt.buf.data() + txt.line_start[l + 1], t);
            const std::string where = "Error in " + tped + ":" + std::to_string(l + 1) + ": ";
            if (t.size() < 4) {
                err.set(l, where + "invalid loci information");
                return;
            }
            al.clear();
            size_t cnt[4] = {0, 0, 0, 0};
            for (size_t k = 4; k < t.size(); ++k)
                for (size_t q = 0; q < t[k].second; ++q) {
                    const char c = t[k].first[q];
                    const int v = c == 'A' ? 0 : c == 'C' ? 1 : c == 'G' ? 2 : c == 'T' ? 3 : -1;
                    if (v < 0) {
                        err.set(l, where + "invalid nucleotide value '" + std::string(1, c) + "'");
                        return;
                    }
                    ++cnt[v];
                    al.push_back((uint8_t)v);
                }
            if (al.size() % 2) {
                err.set(l, where + "odd number of nucleotides");
                return;
            }
            if (al.size() != 2 * n) {
                err.set(l, where + "the number of nucleotides does not match the number of samples");
                return;
            }
            int a1 = -1, a2 = -1;
            for (int i = 0; i < 4; ++i)
                if (cnt[i]) {
                    if (a1 < 0) a1 = i;
                    else if (a2 < 0) a2 = i;
                }
            const int minor = a2 < 0 ? -1 : (cnt[a1] > cnt[a2] ? a2 : a1);
            uint8_t* row = g.codes.data() + snp_of[l] * n;
            for (size_t s = 0; s < n; ++s) row[s] = (uint8_t)((al[2 * s] == minor) + (al[2 * s + 1] == minor));
        }
    });
    if (!err.msg.empty()) return fail(ctx, FIU_ERR_INVALID, err.msg);
    return FIU_OK;
}

bool is_word_char(char c) { return (c >= 'A' && c <= 'Z') || (c >= 'a' && c <= 'z') || (c >= '0' && c <= '9') || c == '_'; }
bool is_alnum(char c) { return (c >= 'A' && c <= 'Z') || (c >= 'a' && c <= 'z') || (c >= '0' && c <= '9'); }

// A column name is a genotype when it is <\w+>_<A|C|G|T> or all alphanumeric.
bool genotype_column(const std::string& w) {
    if (!w.empty() && std::all_of(w.begin(), w.end(), is_alnum)) return true;
    const size_t n = w.size();
    return n >= 3 && w[n - 2] == '_' && (w[n - 1] == 'A' || w[n - 1] == 'C' || w[n - 1] == 'G' || w[n - 1] == 'T') &&
           std::all_of(w.begin(), w.end() - 2, is_word_char);
}

// Integer field as std::stol parses it, the whole token consumed.
bool parse_long(const char* p, size_t len, long& v) {
    const char* e = p + len;
    bool neg = false;
    if (p < e && (*p == '+' || *p == '-')) neg = *p++ == '-';
    if (p == e) return false;
    long x = 0;
    for (; p < e; ++p) {
        if (*p < '0' || *p > '9') return false;
        x = x * 10 + (*p - '0');
    }
    v = neg ? -x : x;
    return true;
}

int read_raw(fiu_ctx* ctx, const std::string& path, int threads, fiu_genotypes& g) {
    Text txt;
    if (!read_file(path, txt.buf)) return fail(ctx, FIU_ERR_INVALID, "Error while opening " + path + ", check file path/permissions");
    split_lines(txt, threads);
    const size_t lines = txt.line_start.size() - 1;
    if (lines == 0) return fail(ctx, FIU_ERR_INVALID, "Error while parsing \"" + path + "\", no phenotype column");
    // header: the \w+ words of the first line
    std::vector<std::string> words;
    {
        const char* p = txt.buf.data();
        const char* e = p + txt.line_start[1];
        while (p < e) {
            while (p < e && !is_word_char(*p)) ++p;
            const char* s = p;
            while (p < e && is_word_char(*p)) ++p;
            if (p > s) words.emplace_back(s, p);
        }
    }
    size_t info = 0;
    const char* names[5] = {"FID", "IID", "PAT", "MAT", "SEX"};
    while (info < 5 && info < words.size() && words[info] == names[info]) ++info;
    const bool has_info = info == 5;
    const std::vector<std::string> cols(words.begin() + (has_info ? 5 : 0), words.end());
    long ph = -1;
    std::vector<int> gcol;  // genotype columns (index within cols)
    for (size_t i = 0; i < cols.size(); ++i) {
        if (cols[i] == "PHENOTYPE" || cols[i] == "Class") {
            if (ph >= 0)
                return fail(ctx, FIU_ERR_INVALID, "Error while parsing \"" + path + "\", multiple phenotype columns found");
            ph = (long)i;
        } else if (genotype_column(cols[i])) {
            gcol.push_back((int)i);
        }
    }
    if (ph < 0) return fail(ctx, FIU_ERR_INVALID, "Error while parsing \"" + path + "\", no phenotype column");
    const size_t ncol = cols.size() + (has_info ? 5 : 0), off = has_info ? 5 : 0;
    // sample rows: non-empty lines after the header
    std::vector<size_t> rows;
    for (size_t l = 1; l < lines; ++l) {
        for (size_t i = txt.line_start[l]; i < txt.line_start[l + 1]; ++i) {
            const char c = txt.buf[i];
            if (!(c == ' ' || c == '\t' || c == '\r' || c == '\n' || c == '\v' || c == '\f')) {
                rows.push_back(l);
                break;
            }
        }
    }
    const size_t n = rows.size(), snps = gcol.size();
    g.samples = n;
    g.snps = snps;
    g.is_case.assign(n, 0);
    try {
        g.codes.assign(snps * n, 0);
    } catch (const std::exception&) {
        return fail(ctx, FIU_ERR_NOMEM, "genotype codes");
    }
    FirstError err;
    parallel_lines(n, threads, [&](size_t a, size_t b) {
        std::vector<std::pair<const char*, size_t>> t;
        for (size_t s = a; s < b; ++s) {
            const size_t l = rows[s];
            if (l >= err.line) return;
            tokens(txt.buf.data() + txt.line_start[l], txt.buf.data() + txt.line_start[l + 1], t);
            if (t.size() != ncol) {
                err.set(l, "Error while parsing \"" + path + "\": ragged row");
                return;
            }
            long v = 0;
            for (size_t i = off; i < ncol; ++i)
                if (!parse_long(t[i].first, t[i].second, v)) {
                    err.set(l, "Error while parsing \"" + path + "\": non-numeric field");
                    return;
                }
            parse_long(t[off + ph].first, t[off + ph].second, v);
            g.is_case[s] = (v + (has_info ? 0 : 1)) != 1;
            for (size_t q = 0; q < snps; ++q) {
                parse_long(t[off + gcol[q]].first, t[off + gcol[q]].second, v);
                g.codes[q * n + s] = (uint8_t)v;
            }
        }
    });
    if (!err.msg.empty()) return fail(ctx, FIU_ERR_INVALID, err.msg);
    return FIU_OK;
}

// One warp per (SNP, class): row set of the reference layout from the codes.
__global__ void pack_kernel(const uint8_t* __restrict__ codes, const int* __restrict__ idx, int n_cases, int n_ctrls,
                            long long samples, int snps, int cw, int tw, uint64_t* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long wi = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); wi < 2ll * snps; wi += warps) {
        const int snp = (int)(wi >> 1), cls = (int)(wi & 1);
        const int cnt = cls ? n_ctrls : n_cases, W = cls ? tw : cw;
        const int* ix = idx + (cls ? n_cases : 0);
        const uint8_t* row = codes + (size_t)snp * samples;
        uint64_t* o = out + (size_t)snp * 3 * (cw + tw) + (cls ? 3 * (size_t)cw : 0);
        for (int w = 0; w < W; ++w) {
            const int s0 = 64 * w + lane, s1 = s0 + 32;
            const int c0 = s0 < cnt ? __ldg(row + __ldg(ix + s0)) : 3;
            const int c1 = s1 < cnt ? __ldg(row + __ldg(ix + s1)) : 3;
            const int valid = min(64, max(0, cnt - 64 * w));  // samples in this word
#pragma unroll
            for (int g = 0; g < 3; ++g) {
                const unsigned b0 = __ballot_sync(0xffffffffu, c0 == g), b1 = __ballot_sync(0xffffffffu, c1 == g);
                // sample 64 w + b at bit 63 - b, then right-aligned when the word is partial
                uint64_t v = ((uint64_t)__brev(b0) << 32) | (uint64_t)__brev(b1);
                if (valid == 0) v = 0;
                else if (valid < 64) v >>= (64 - valid);
                if (lane == 0) o[(size_t)g * W + w] = v;
            }
        }
    }
}

}  // namespace

extern "C" {

int fiu_read_genotypes(fiu_ctx* ctx, const char* f1, const char* f2, int threads, fiu_genotypes** out) {
    if (!out || !f1) return FIU_ERR_INVALID;
    *out = nullptr;
    if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    auto* g = new (std::nothrow) fiu_genotypes;
    if (!g) return fail(ctx, FIU_ERR_NOMEM, "host allocation");
    int rc = FIU_OK;
    const std::string a = f1, b = f2 ? f2 : "";
    try {
        if (b.empty()) {
            if (ext_of(a) == ".raw") rc = read_raw(ctx, a, threads, *g);
            else rc = fail(ctx, FIU_ERR_INVALID, "Unrecognized input file extension " + ext_of(a));
        } else {
            const std::string e1 = ext_of(a), e2 = ext_of(b);
            if (e1 != ".tped" && e1 != ".tfam") rc = fail(ctx, FIU_ERR_INVALID, "Unrecognized input file extension " + e1);
            else if (e1 == e2 || (e2 != ".tped" && e2 != ".tfam"))
                rc = fail(ctx, FIU_ERR_INVALID, "Expecting a tfam file after \"" + a + "\", but found a " + e2);
            else rc = e1 == ".tped" ? read_tped(ctx, a, b, threads, *g) : read_tped(ctx, b, a, threads, *g);
        }
    } catch (const std::exception& e) {
        rc = fail(ctx, FIU_ERR_NOMEM, std::string("reading genotypes: ") + e.what());
    }
    if (rc) {
        delete g;
        return rc;
    }
    *out = g;
    return FIU_OK;
}

int fiu_genotypes_info(const fiu_genotypes* g, uint64_t* snps, uint64_t* samples, const uint8_t** codes,
                       const uint8_t** is_case) {
    if (!g) return FIU_ERR_INVALID;
    if (snps) *snps = g->snps;
    if (samples) *samples = g->samples;
    if (codes) *codes = g->codes.data();
    if (is_case) *is_case = g->is_case.data();
    return FIU_OK;
}

void fiu_genotypes_free(fiu_genotypes* g) { delete g; }

int fiu_dataset_upload_genotypes(fiu_ctx* ctx, const uint8_t* codes, const uint8_t* is_case, uint64_t snps,
                                 uint64_t samples, fiu_resident** out) {
    if (!ctx || !out) return FIU_ERR_INVALID;
    Scope scope(ctx);
    *out = nullptr;
    if (!codes || !is_case) return fail(ctx, FIU_ERR_INVALID, "null genotype codes");
    if (samples > 0x7fffffffull) return fail(ctx, FIU_ERR_INVALID, "too many samples");
    std::vector<int> idx(samples);
    uint64_t cases = 0;
    for (uint64_t s = 0; s < samples; ++s)
        if (is_case[s]) idx[cases++] = (int)s;
    uint64_t c2 = cases;
    for (uint64_t s = 0; s < samples; ++s)
        if (!is_case[s]) idx[c2++] = (int)s;
    const uint64_t ctrls = samples - cases, cw = (cases + 63) / 64, tw = (ctrls + 63) / 64;
    int rc = check_sizes(ctx, snps, cases, ctrls, cw, tw);
    if (rc) return rc;
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    fiu_resident* r = nullptr;
    if ((rc = new_resident(ctx, snps, cases, ctrls, cw, tw, &r))) return rc;
    cudaStream_t s = ctx->stream;
    uint8_t* dc = nullptr;
    int* di = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&dc, snps * samples, s);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&di, samples * sizeof(int) + 4, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dc, codes, snps * samples, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && samples) e = cudaMemcpyAsync(di, idx.data(), samples * sizeof(int), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        const long long warps = 2ll * (long long)snps;
        const int grid = (int)std::min<long long>((warps + 7) / 8, 8ll * ctx->sms);
        pack_kernel<<<grid, 256, 0, s>>>(dc, di, (int)cases, (int)ctrls, (long long)samples, (int)snps, (int)cw,
                                         (int)tw, r->ref);
        count_launch();
        e = cudaGetLastError();
    }
    if (dc) cudaFreeAsync(dc, s);
    if (di) cudaFreeAsync(di, s);
    if (e != cudaSuccess) {
        cudaStreamSynchronize(s);
        fiu_dataset_free(ctx, r);
        return cuda_fail(ctx, e, "genotype packing");
    }
    if ((rc = finish_resident(ctx, r))) return rc;
    *out = r;
    return FIU_OK;
}

int fiu_dataset_packed(fiu_ctx* ctx, const fiu_resident* res, fiu_dataset* desc, uint64_t* data) {
    if (!ctx || !res) return FIU_ERR_INVALID;
    Scope scope(ctx);
    if (desc) {
        desc->data = nullptr;
        desc->snps = (uint64_t)res->d.snps;
        desc->cases = (uint64_t)res->d.n_cases;
        desc->ctrls = (uint64_t)res->d.n_ctrls;
        desc->cases_words = (uint64_t)res->d.cw;
        desc->ctrls_words = (uint64_t)res->d.tw;
    }
    if (!data) return FIU_OK;
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    const size_t words = (size_t)res->d.snps * 3 * (size_t)(res->d.cw + res->d.tw);
    CK(cudaMemcpyAsync(data, res->ref, words * 8, cudaMemcpyDeviceToHost, ctx->stream), "packed data");
    CK(cudaStreamSynchronize(ctx->stream), "packed data");
    return FIU_OK;
}

}  // extern "C"
