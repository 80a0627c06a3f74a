// Test driver of the LevelCellArray layout builder of the restart files
// (samurai_gb300/csrc/sg_csr.hpp).  Reads "dim n" and n records
// "start end y [z] index" (x-intervals row by row, z outer and y inner) from
// standard input and prints, per dimension d, "ivd" then "start,end,index" of
// every interval, and per offsets array "offd" then its entries.
//   csr_tool decode <level>           also decodes the layout back (decode_csr) and prints
//                                     "dec <code>" and "cells x,y[,z] ..."
//   csr_tool fuzz <level> <seed> <n>  n corrupted copies of the layout (intervals and offsets
//                                     overwritten), each decoded; prints "ok outside inconsistent"
//   csr_tool raw <level>              reads a layout as written in a file instead: "dim", then per
//                                     dimension d a count and "start end index" records, then per
//                                     offsets array a count and its entries; prints "dec <code> <cells>"
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "../../samurai_gb300/csrc/sg_csr.hpp"

// decode_csr on corrupted copies: it must return on each, and a layout it accepts gives cells inside the box
// (the test builds this under the address and undefined-behaviour sanitizers)
static int fuzz(int dim, int level, const sg::csr::LevelCSR& good, unsigned long long seed, int n)
{
    unsigned long long x = seed * 0x9E3779B97F4A7C15ull + 1;
    auto rnd             = [&]
    {
        x ^= x << 13;
        x ^= x >> 7;
        x ^= x << 17;
        return x;
    };
    const long long vals[] = {-1, 0, 1, 2, 1LL << 31, -(1LL << 31), 1LL << 40, -(1LL << 62) - 5, (1LL << 62) + 5, 1 << level, (1 << level) + 1};
    int cnt[3] = {0, 0, 0};
    for (int it = 0; it < n; ++it)
    {
        sg::csr::LevelCSR c = good;
        for (int m = 0, nm = 1 + static_cast<int>(rnd() % 3); m < nm; ++m)
        {
            const long long v = (rnd() & 1) ? vals[rnd() % 11] : static_cast<long long>(rnd() % 64) - 8;
            const int which   = static_cast<int>(rnd() % (dim == 3 ? 5 : 3));
            if (which < dim && !c.iv[which].empty())
            {
                auto& r      = c.iv[which][rnd() % c.iv[which].size()];
                const int fld = static_cast<int>(rnd() % 3);
                if (fld == 0)
                {
                    r.start = static_cast<int32_t>(v);
                }
                else if (fld == 1)
                {
                    r.end = static_cast<int32_t>(v);
                }
                else
                {
                    r.index = v;
                }
            }
            else if (which >= dim && !c.off[which - dim].empty())
            {
                c.off[which - dim][rnd() % c.off[which - dim].size()] = static_cast<uint64_t>(v);
            }
            else if (!c.off[0].empty())
            {
                c.off[0].resize(rnd() % c.off[0].size());
            }
        }
        std::vector<int> co;
        const auto d = sg::csr::decode_csr(dim, level, c, co);
        ++cnt[static_cast<int>(d)];
        if (d == sg::csr::Decode::ok)
        {
            for (int v : co)
            {
                if (v < 0 || v >= (1 << level))
                {
                    std::fprintf(stderr, "iteration %d: a decoded cell outside the box\n", it);
                    return 4;
                }
            }
        }
    }
    std::printf("%d %d %d\n", cnt[0], cnt[1], cnt[2]);
    return 0;
}

// a layout given array by array, as a restart file holds it
static int raw(int level)
{
    int dim = 0;
    if (std::scanf("%d", &dim) != 1 || (dim != 2 && dim != 3))
    {
        return 2;
    }
    sg::csr::LevelCSR c;
    for (int d = 0; d < dim; ++d)
    {
        long long n = 0;
        if (std::scanf("%lld", &n) != 1 || n < 0)
        {
            return 2;
        }
        for (long long k = 0; k < n; ++k)
        {
            long long s = 0, e = 0, i = 0;
            if (std::scanf("%lld %lld %lld", &s, &e, &i) != 3)
            {
                return 2;
            }
            sg::csr::IntervalRec r{};
            r.start = static_cast<int32_t>(s);
            r.end   = static_cast<int32_t>(e);
            r.step  = 1;
            r.index = i;
            c.iv[d].push_back(r);
        }
    }
    for (int d = 0; d + 1 < dim; ++d)
    {
        long long n = 0;
        if (std::scanf("%lld", &n) != 1 || n < 0)
        {
            return 2;
        }
        for (long long k = 0; k < n; ++k)
        {
            unsigned long long v = 0;
            if (std::scanf("%llu", &v) != 1)
            {
                return 2;
            }
            c.off[d].push_back(v);
        }
    }
    std::vector<int> co;
    const auto d = sg::csr::decode_csr(dim, level, c, co);
    std::printf("dec %d %zu\n", static_cast<int>(d), co.size() / static_cast<size_t>(dim));
    return 0;
}

int main(int argc, char** argv)
{
    const std::string mode = argc >= 2 ? argv[1] : "";
    if (mode == "raw" && argc >= 3)
    {
        return raw(std::atoi(argv[2]));
    }
    int dim       = 0;
    long long n   = 0;
    if (std::scanf("%d %lld", &dim, &n) != 2 || (dim != 2 && dim != 3) || n < 0)
    {
        return 2;
    }
    std::vector<long long> rows(static_cast<size_t>(n) * (dim + 2));
    for (auto& v : rows)
    {
        if (std::scanf("%lld", &v) != 1)
        {
            return 2;
        }
    }
    sg::csr::LevelCSR c;
    sg::csr::build_csr(dim, rows, c);
    if (mode == "fuzz" && argc >= 5)
    {
        return fuzz(dim, std::atoi(argv[2]), c, std::strtoull(argv[3], nullptr, 10), std::atoi(argv[4]));
    }
    for (int d = 0; d < dim; ++d)
    {
        std::printf("iv%d", d);
        for (const auto& r : c.iv[d])
        {
            std::printf(" %d,%d,%lld", r.start, r.end, static_cast<long long>(r.index));
        }
        std::printf("\n");
    }
    for (int d = 0; d < dim - 1; ++d)
    {
        std::printf("off%d", d);
        for (auto v : c.off[d])
        {
            std::printf(" %llu", static_cast<unsigned long long>(v));
        }
        std::printf("\n");
    }
    if (mode == "decode" && argc >= 3)
    {
        std::vector<int> co;
        const auto d = sg::csr::decode_csr(dim, std::atoi(argv[2]), c, co);
        std::printf("dec %d\ncells", static_cast<int>(d));
        for (size_t k = 0; k < co.size(); k += static_cast<size_t>(dim))
        {
            std::printf(dim == 2 ? " %d,%d" : " %d,%d,%d", co[k], co[k + 1], dim == 3 ? co[k + 2] : 0);
        }
        std::printf("\n");
    }
    return 0;
}
