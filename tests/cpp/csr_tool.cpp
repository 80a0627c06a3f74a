// Test driver of the LevelCellArray layout builder of the restart files
// (samurai_gb300/csrc/sg_csr.hpp).  Reads "dim n" and n records
// "start end y [z] index" (x-intervals row by row, z outer and y inner) from
// standard input and prints, per dimension d, "ivd" then "start,end,index" of
// every interval, and per offsets array "offd" then its entries.
#include <cstdio>
#include <vector>

#include "../../samurai_gb300/csrc/sg_csr.hpp"

int main()
{
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
    return 0;
}
