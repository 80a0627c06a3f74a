// Test driver of the HDF5 layer of libsamurai_gpu (samurai_gb300/csrc/sg_h5.hpp).
//   h5_tool write <file.h5>            writes a fixed set of groups and datasets
//   h5_tool read <file.h5> <path>      prints "class size signed shape..." then the values
//   h5_tool exists <file.h5> <path>    prints 1 or 0
//   h5_tool toomany <file.h5>          a group of 300 members: exits 3 (refused)
#include <cinttypes>
#include <cstdio>
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

int main(int argc, char** argv)
{
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
