/**
 * @file Result.h
 * @brief Result<U,V> of the host-side C++ mirror: a combination and its value,
 * ordered by value only, with the reference's text form and binary
 * serialisation (include/fiuncho/utils/Result.h:17-70 of the reference).
 */
#ifndef FIUNCHO_RESULT_H
#define FIUNCHO_RESULT_H

#include <istream>
#include <ostream>
#include <sstream>
#include <string>
#include <vector>

template <typename U, typename V> class Result
{
  public:
    Result() : val(0) {}

    bool operator<(const Result &o) const { return val < o.val; }
    bool operator>(const Result &o) const { return o.val < val; }
    bool operator<=(const Result &o) const { return !(o.val < val); }
    bool operator>=(const Result &o) const { return !(val < o.val); }
    bool operator==(const Result &o) const { return val == o.val && combination == o.combination; }
    bool operator!=(const Result &o) const { return !(*this == o); }

    /** "i j ... val" with the stream's default 6 significant digits. */
    std::string str() const
    {
        std::ostringstream s;
        for (const U &i : combination) s << i << ' ';
        s << val;
        return s.str();
    }

    /** size (size_t), indices (U), value (V), native byte order. */
    static std::ostream &serialize(std::ostream &os, const Result &r)
    {
        const size_t n = r.combination.size();
        os.write(reinterpret_cast<const char *>(&n), sizeof n);
        os.write(reinterpret_cast<const char *>(r.combination.data()), n * sizeof(U));
        os.write(reinterpret_cast<const char *>(&r.val), sizeof(V));
        return os;
    }

    static std::istream &deserialize(std::istream &is, Result &r)
    {
        size_t n = 0;
        is.read(reinterpret_cast<char *>(&n), sizeof n);
        r.combination.resize(n);
        is.read(reinterpret_cast<char *>(r.combination.data()), n * sizeof(U));
        is.read(reinterpret_cast<char *>(&r.val), sizeof(V));
        return is;
    }

    std::vector<U> combination;
    V val;
};

#endif
