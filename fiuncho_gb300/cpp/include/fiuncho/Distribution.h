/**
 * @file Distribution.h
 * @brief Distribution<T> of the host-side C++ mirror: the k-combinations of n
 * in lexicographic order, of which this worker owns ranks offset,
 * offset + step, ... (the reference's include/fiuncho/Distribution.h:24-203).
 * Iteration unranks each owned rank directly.
 */
#ifndef FIUNCHO_DISTRIBUTION_H
#define FIUNCHO_DISTRIBUTION_H

#include <cstdint>
#include <type_traits>
#include <vector>

template <typename T> class Distribution
{
    static unsigned long long binom(long long n, long long k)
    {
        if (k < 0 || n < k) return 0;
        if (k > n - k) k = n - k;
        unsigned __int128 r = 1;
        for (long long i = 1; i <= k; ++i) {
            r = r * (unsigned long long)(n - k + i) / (unsigned long long)i;
            if (r >> 63) return 1ull << 63;
        }
        return (unsigned long long)r;
    }

  public:
    const T n, k, step, offset;

    Distribution(const T &n, const T &k, const T &step, const T &offset) : n(n), k(k), step(step), offset(offset)
    {
        static_assert(std::is_signed<T>::value, "Distribution template parameter requires a signed type");
    }

    Distribution<T> layer(const T s, const T o) const { return Distribution<T>(n, k, step * s, offset * s + o); }

    /** Number of combinations in total (owned or not). */
    unsigned long long total() const { return binom(n, k); }

    class const_iterator
    {
        friend class Distribution<T>;
        const Distribution<T> *d;
        unsigned long long rank;
        std::vector<T> c;

        void fill()
        {
            c.assign(d->k, 0);
            if (rank >= d->total()) {
                if (d->k > 0) c[0] = d->n;
                return;
            }
            unsigned long long r = rank;
            T start = 0;
            for (T t = 0; t < d->k; ++t) {
                // smallest first element whose block contains rank r
                for (T x = start;; ++x) {
                    const unsigned long long block = binom(d->n - 1 - x, d->k - 1 - t);
                    if (r < block) {
                        c[t] = x;
                        start = x + 1;
                        break;
                    }
                    r -= block;
                }
            }
        }

      public:
        const_iterator(const Distribution<T> &dist, unsigned long long r) : d(&dist), rank(r) { fill(); }
        const std::vector<T> &operator*() const { return c; }
        const std::vector<T> *operator->() const { return &c; }
        const T &operator[](size_t i) const { return c[i]; }
        const_iterator &operator++()
        {
            rank += (unsigned long long)d->step;
            fill();
            return *this;
        }
        bool operator<(const const_iterator &o) const { return rank < o.rank && rank < d->total(); }
    };

    const_iterator begin() const { return const_iterator(*this, (unsigned long long)offset); }
    const_iterator end() const { return const_iterator(*this, total()); }
};

#endif
