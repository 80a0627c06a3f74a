// Test driver of the HDF5 layer of libsamurai_gpu (samurai_gb300/csrc/sg_h5.hpp).
//   h5_tool write <file.h5>            writes a fixed set of groups and datasets
//   h5_tool read <file.h5> <path>      prints "class size signed shape..." then the values
//   h5_tool exists <file.h5> <path>    prints 1 or 0
//   h5_tool toomany <file.h5>          a group of 300 members: exits 3 (refused)
//   h5_tool fuzz <file.h5> <seed> <n>  n corrupted copies of <file.h5>, each opened and read along
//                                      every path of the write mode; prints "opened read_ok read_err"
#include <cinttypes>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../samurai_gb300/csrc/sg_h5.hpp"

namespace h5 = sg::h5;

static int write_file(const char* name)
{
    h5::Writer w;
    const uint64_t n_process = 1;
    w.add("/n_process", h5::Kind::U64, {}, &n_process);
    std::vector<double> pts = {0., 0., 0., 0.5, 0., 0., 0.5, 0.25, 0., -1.5e300, 3.25, 1e-300};
    w.add("/mesh/points", h5::Kind::F64, {4, 3}, pts.data());
    std::vector<uint64_t> conn = {0, 1, 2, 3, 3, 2, 1, 0};
    w.add("/mesh/connectivity", h5::Kind::U64, {2, 4}, conn.data());
    std::vector<int64_t> i64 = {-5, 7, -9000000000LL};
    w.add("/mesh/fields/signed", h5::Kind::I64, {3}, i64.data());
    std::vector<int32_t> i32 = {-1, 2147483647};
    w.add("/mesh/fields/small", h5::Kind::I32, {2}, i32.data());
    struct Interval
    {
        int32_t start, end, step;
        int32_t pad;
        int64_t index;
    };
    Interval iv[2] = {{-3, 5, 1, 0, 17}, {8, 9, 1, 0, -8}};
    w.add("/mesh/level/4/dim/0/intervals/data", h5::Kind::Interval, {2}, iv);
    // a group with more members than one symbol table node holds
    for (int k = 0; k < 21; ++k)
    {
        const double v = k * 0.5;
        w.add("/many/m" + std::to_string(k), h5::Kind::F64, {}, &v);
    }
    w.add("/empty", h5::Kind::F64, {0}, nullptr);
    std::string err;
    if (!w.save(name, err))
    {
        std::fprintf(stderr, "%s\n", err.c_str());
        return 1;
    }
    return 0;
}

static int read_path(const char* name, const char* path)
{
    h5::Reader r;
    std::string err;
    h5::Array a;
    if (!r.open(name, err) || !r.read(path, a, err))
    {
        std::fprintf(stderr, "%s\n", err.c_str());
        return 1;
    }
    std::printf("%d %zu %d", a.cls, a.size, a.is_signed ? 1 : 0);
    for (auto s : a.shape)
    {
        std::printf(" %" PRIu64, s);
    }
    std::printf("\n");
    const uint64_t n = a.count();
    for (uint64_t k = 0; k < n; ++k)
    {
        const uint8_t* p = a.bytes.data() + k * a.size;
        if (a.cls == 1)
        {
            double v;
            std::memcpy(&v, p, 8);
            std::printf("%.17g\n", v);
        }
        else if (a.cls == 0 && a.size == 8)
        {
            int64_t v;
            std::memcpy(&v, p, 8);
            std::printf(a.is_signed ? "%" PRId64 "\n" : "%" PRIu64 "\n", v);
        }
        else if (a.cls == 0 && a.size == 4)
        {
            int32_t v;
            std::memcpy(&v, p, 4);
            std::printf(a.is_signed ? "%d\n" : "%u\n", v);
        }
        else if (a.cls == 6)
        {
            // members in name order with their offsets, then the record as int32 start/end/step and int64 index
            int32_t s, e, st;
            int64_t ix;
            std::memcpy(&s, p + a.members.at("start"), 4);
            std::memcpy(&e, p + a.members.at("end"), 4);
            std::memcpy(&st, p + a.members.at("step"), 4);
            std::memcpy(&ix, p + a.members.at("index"), 8);
            std::printf("%d %d %d %" PRId64 "\n", s, e, st, ix);
        }
    }
    return 0;
}

// a group of 300 members: beyond one B-tree node, refused
static int too_many(const char* name)
{
    h5::Writer w;
    for (int k = 0; k < 300; ++k)
    {
        const double v = k;
        w.add("/g/m" + std::to_string(k), h5::Kind::F64, {}, &v);
    }
    std::string err;
    if (w.save(name, err))
    {
        return 0;
    }
    std::fprintf(stderr, "%s\n", err.c_str());
    return 3;
}

// Corrupted copies: truncations, flipped bits, overwritten 16-bit and 64-bit fields (offsets, sizes,
// counts).  The reader must return on each, true or false, and what it returns as read must be
// consistent; the test builds this tool with the address and undefined-behaviour sanitizers, which
// turn any read outside the buffer into a failure.
static int fuzz(const char* name, uint64_t seed, int n)
{
    std::vector<uint8_t> orig;
    {
        FILE* f = std::fopen(name, "rb");
        if (!f)
        {
            return 1;
        }
        uint8_t buf[4096];
        size_t got;
        while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0)
        {
            orig.insert(orig.end(), buf, buf + got);
        }
        std::fclose(f);
    }
    if (orig.size() < 64)
    {
        return 1;
    }
    const char* paths[] = {"/n_process",    "/mesh/points", "/mesh/connectivity", "/mesh/fields/signed", "/mesh/fields/small",
                           "/mesh/level/4/dim/0/intervals/data", "/many/m0", "/many/m20", "/empty", "/nothing", "/mesh/nothing/x"};
    uint64_t x = seed * 0x9E3779B97F4A7C15ull + 1;
    auto rnd   = [&]
    {
        x ^= x << 13;
        x ^= x >> 7;
        x ^= x << 17;
        return x;
    };
    const std::string tmp = std::string(name) + ".fuzz";
    int opened = 0, read_ok = 0, read_err = 0;
    for (int it = 0; it < n; ++it)
    {
        std::vector<uint8_t> b = orig;
        const uint64_t kind    = rnd() % 4;
        if (kind == 0)
        {
            b.resize(rnd() % b.size());
        }
        else if (kind == 1)
        {
            for (uint64_t k = 0, nk = 1 + rnd() % 8; k < nk; ++k)
            {
                b[rnd() % b.size()] ^= static_cast<uint8_t>(1u << (rnd() % 8));
            }
        }
        else if (kind == 2)
        {
            const size_t at      = (rnd() & 1) ? (rnd() % (b.size() / 8)) * 8 : rnd() % (b.size() - 8);
            const uint64_t cands[] = {0, ~uint64_t(0), rnd(), b.size(), b.size() - 1, uint64_t(1) << 40, rnd() % b.size()};
            const uint64_t v     = cands[rnd() % 7];
            std::memcpy(&b[at], &v, 8);
        }
        else
        {
            const size_t at = rnd() % (b.size() - 2);
            const uint16_t v = static_cast<uint16_t>(rnd());
            std::memcpy(&b[at], &v, 2);
        }
        FILE* f = std::fopen(tmp.c_str(), "wb");
        if (!f || std::fwrite(b.data(), 1, b.size(), f) != b.size())
        {
            return 1;
        }
        std::fclose(f);
        h5::Reader r;
        std::string err;
        if (!r.open(tmp, err))
        {
            continue;
        }
        ++opened;
        for (const char* p : paths)
        {
            h5::Array a;
            std::string e;
            if (r.read(p, a, e))
            {
                ++read_ok;
                if (a.bytes.size() != a.count() * a.size)
                {
                    std::fprintf(stderr, "iteration %d: %s: %zu bytes for %" PRIu64 " elements of %zu\n", it, p, a.bytes.size(), a.count(), a.size);
                    return 4;
                }
                for (auto& m : a.members)
                {
                    if (m.second + a.member_size.at(m.first) > a.size)
                    {
                        std::fprintf(stderr, "iteration %d: %s: member %s outside the record\n", it, p, m.first.c_str());
                        return 4;
                    }
                }
            }
            else
            {
                ++read_err;
                if (e.empty())
                {
                    std::fprintf(stderr, "iteration %d: %s: refused without a message\n", it, p);
                    return 4;
                }
            }
            r.exists(p);
        }
    }
    std::remove(tmp.c_str());
    std::printf("%d %d %d\n", opened, read_ok, read_err);
    return 0;
}

int main(int argc, char** argv)
{
    if (argc >= 5 && std::string(argv[1]) == "fuzz")
    {
        return fuzz(argv[2], std::strtoull(argv[3], nullptr, 10), std::atoi(argv[4]));
    }
    if (argc >= 3 && std::string(argv[1]) == "toomany")
    {
        return too_many(argv[2]);
    }
    if (argc >= 3 && std::string(argv[1]) == "write")
    {
        return write_file(argv[2]);
    }
    if (argc >= 4 && std::string(argv[1]) == "read")
    {
        return read_path(argv[2], argv[3]);
    }
    if (argc >= 4 && std::string(argv[1]) == "exists")
    {
        h5::Reader r;
        std::string err;
        if (!r.open(argv[2], err))
        {
            std::fprintf(stderr, "%s\n", err.c_str());
            return 1;
        }
        std::printf("%d\n", r.exists(argv[3]) ? 1 : 0);
        return 0;
    }
    std::fprintf(stderr, "usage: h5_tool write <file> | read <file> <path> | exists <file> <path>\n");
    return 2;
}
