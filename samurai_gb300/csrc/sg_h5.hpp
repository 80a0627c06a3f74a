// Minimal HDF5 writer and reader (no libhdf5), for the files samurai writes
// on this path: save() (io/hdf5.hpp:682-937: /mesh/points, /mesh/connectivity,
// /mesh/fields/<name>) and the restart dump()/load() (io/restart.hpp:50-463).
//
// Writer: the file layout the HDF5 library produces by default for those
// calls -- superblock version 0, version 1 object headers, groups as symbol
// tables (a version 1 B-tree of type 0 with one level of symbol table nodes
// and a local heap of names), datasets with a version 1 dataspace, a version
// 2 fill value message and contiguous storage (layout message version 3).
// Datatypes: 32/64-bit integers, IEEE binary64 and samurai's Interval
// compound {start, end, step: int32; index: int64} (io/restart.hpp:31-47).
// Layout rules followed (HDF5 file format specification, version 2.0+):
// every structure starts on an 8-byte boundary; group members are sorted by
// name, at most 2 * leaf_k = 8 per symbol table node; the B-tree key left of
// child i is the last name of child i-1 (the empty name for i = 0).
//
// Reader: superblock 0, version 1 object headers with continuation
// blocks, symbol-table groups (B-trees of any depth), dataspace versions 1/2,
// fixed-point / floating-point / compound (versions 1-3) datatypes,
// contiguous and compact layouts without filters.  Anything else is reported
// as an error, never guessed.
#pragma once

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace sg
{
    namespace h5
    {
        constexpr uint64_t UNDEF = ~uint64_t(0);

        enum class Kind
        {
            U64,
            I64,
            I32,
            F64,
            Interval // samurai::Interval<int, long long>: 24 bytes
        };

        inline size_t kind_size(Kind k)
        {
            switch (k)
            {
                case Kind::I32:
                    return 4;
                case Kind::Interval:
                    return 24;
                default:
                    return 8;
            }
        }

        // --------------------------------------------------------------- writer
        class Writer
        {
          public:

            // path: "/a/b/name"; shape empty = scalar
            void add(const std::string& path, Kind kind, const std::vector<uint64_t>& shape, const void* data)
            {
                Entry e;
                e.kind  = kind;
                e.shape = shape;
                uint64_t n = 1;
                for (auto s : shape)
                {
                    n *= s;
                }
                e.bytes.resize(static_cast<size_t>(n) * kind_size(kind));
                if (!e.bytes.empty())
                {
                    std::memcpy(e.bytes.data(), data, e.bytes.size());
                }
                Group* g      = &m_root;
                size_t p      = 1;
                std::string nm;
                for (;;)
                {
                    const size_t q = path.find('/', p);
                    if (q == std::string::npos)
                    {
                        nm = path.substr(p);
                        break;
                    }
                    auto& sub = g->groups[path.substr(p, q - p)];
                    if (!sub)
                    {
                        sub = std::make_unique<Group>();
                    }
                    g = sub.get();
                    p = q + 1;
                }
                g->datasets[nm] = std::move(e);
            }

            bool save(const std::string& filename, std::string& err)
            {
                m_out.assign(96, 0);
                m_too_many = false;
                const uint64_t root = emit_group(m_root);
                if (m_too_many)
                {
                    err = "a group has more than 256 members, more than one B-tree node holds";
                    return false;
                }
                // superblock version 0
                std::memcpy(m_out.data(), "\x89HDF\r\n\x1a\n", 8);
                m_out[13] = 8;                   // size of offsets
                m_out[14] = 8;                   // size of lengths
                put16(16, 4);                    // group leaf node K
                put16(18, 16);                   // group internal node K
                put64(24, 0);                    // base address
                put64(32, UNDEF);                // free-space info
                put64(40, m_out.size());         // end of file address
                put64(48, UNDEF);                // driver information block
                put64(56, 0);                    // root entry: link name offset
                put64(64, root);                 //   object header
                put32(72, 1);                    //   cache type 1: B-tree and heap addresses
                put64(80, m_root.btree);
                put64(88, m_root.heap);
                FILE* f = std::fopen(filename.c_str(), "wb");
                if (!f)
                {
                    err = "cannot open " + filename + " for writing";
                    return false;
                }
                const bool ok = std::fwrite(m_out.data(), 1, m_out.size(), f) == m_out.size();
                if (std::fclose(f) != 0 || !ok)
                {
                    err = "cannot write " + filename;
                    return false;
                }
                return true;
            }

          private:

            struct Entry
            {
                Kind kind;
                std::vector<uint64_t> shape;
                std::vector<uint8_t> bytes;
            };

            struct Group
            {
                std::map<std::string, std::unique_ptr<Group>> groups;
                std::map<std::string, Entry> datasets;
                uint64_t btree = 0, heap = 0;
            };

            void put8(uint64_t at, uint8_t v)
            {
                m_out[at] = v;
            }

            void put16(uint64_t at, uint16_t v)
            {
                for (int k = 0; k < 2; ++k)
                {
                    m_out[at + k] = static_cast<uint8_t>(v >> (8 * k));
                }
            }

            void put32(uint64_t at, uint32_t v)
            {
                for (int k = 0; k < 4; ++k)
                {
                    m_out[at + k] = static_cast<uint8_t>(v >> (8 * k));
                }
            }

            void put64(uint64_t at, uint64_t v)
            {
                for (int k = 0; k < 8; ++k)
                {
                    m_out[at + k] = static_cast<uint8_t>(v >> (8 * k));
                }
            }

            // reserve n zero bytes at the next 8-byte boundary
            uint64_t alloc(uint64_t n)
            {
                const uint64_t at = (m_out.size() + 7) & ~uint64_t(7);
                m_out.resize(at + n, 0);
                return at;
            }

            // datatype message body for a scalar type (class 0 or 1, version 1)
            static std::vector<uint8_t> type_body(Kind k)
            {
                std::vector<uint8_t> b;
                auto u16 = [&](uint16_t v) { b.push_back(uint8_t(v)); b.push_back(uint8_t(v >> 8)); };
                auto u32 = [&](uint32_t v) { for (int i = 0; i < 4; ++i) b.push_back(uint8_t(v >> (8 * i))); };
                switch (k)
                {
                    case Kind::F64:
                        b = {0x11, 0x20, 0x3f, 0x00}; // version 1 floating point; LE, implied MSB, sign at bit 63
                        u32(8);
                        u16(0);
                        u16(64);
                        b.push_back(52); // exponent location
                        b.push_back(11); // exponent size
                        b.push_back(0);  // mantissa location
                        b.push_back(52); // mantissa size
                        u32(1023);       // exponent bias
                        break;
                    case Kind::I32:
                        b = {0x10, 0x08, 0x00, 0x00}; // version 1 fixed point, LE, signed
                        u32(4);
                        u16(0);
                        u16(32);
                        break;
                    case Kind::I64:
                        b = {0x10, 0x08, 0x00, 0x00};
                        u32(8);
                        u16(0);
                        u16(64);
                        break;
                    default: // U64
                        b = {0x10, 0x00, 0x00, 0x00};
                        u32(8);
                        u16(0);
                        u16(64);
                        break;
                }
                return b;
            }

            // samurai's Interval compound (io/restart.hpp:31-47), version 1 compound members
            static std::vector<uint8_t> interval_body()
            {
                std::vector<uint8_t> b = {0x16, 4, 0, 0}; // version 1 compound, 4 members
                auto u32 = [&](uint32_t v) { for (int i = 0; i < 4; ++i) b.push_back(uint8_t(v >> (8 * i))); };
                u32(24);
                const char* names[4]  = {"start", "end", "step", "index"};
                const uint32_t off[4] = {0, 4, 8, 16};
                for (int m = 0; m < 4; ++m)
                {
                    const size_t n = std::strlen(names[m]) + 1;
                    for (size_t i = 0; i < ((n + 7) & ~size_t(7)); ++i)
                    {
                        b.push_back(i < n - 1 ? uint8_t(names[m][i]) : 0);
                    }
                    u32(off[m]);
                    b.push_back(0); // dimensionality
                    b.insert(b.end(), 3 + 4 + 4 + 16, 0);
                    auto t = type_body(m < 3 ? Kind::I32 : Kind::I64);
                    b.insert(b.end(), t.begin(), t.end());
                }
                return b;
            }

            // version 1 object header holding the given messages (type, body)
            uint64_t emit_header(const std::vector<std::pair<uint16_t, std::vector<uint8_t>>>& msgs)
            {
                uint64_t body = 0;
                for (auto& m : msgs)
                {
                    body += 8 + ((m.second.size() + 7) & ~size_t(7));
                }
                const uint64_t at = alloc(16 + body);
                put8(at, 1);
                put16(at + 2, static_cast<uint16_t>(msgs.size()));
                put32(at + 4, 1);
                put32(at + 8, static_cast<uint32_t>(body));
                uint64_t p = at + 16;
                for (auto& m : msgs)
                {
                    const uint64_t sz = (m.second.size() + 7) & ~size_t(7);
                    put16(p, m.first);
                    put16(p + 2, static_cast<uint16_t>(sz));
                    std::memcpy(&m_out[p + 8], m.second.data(), m.second.size());
                    p += 8 + sz;
                }
                return at;
            }

            uint64_t emit_dataset(const Entry& e)
            {
                uint64_t data = UNDEF;
                if (!e.bytes.empty())
                {
                    data = alloc(e.bytes.size());
                    std::memcpy(&m_out[data], e.bytes.data(), e.bytes.size());
                }
                std::vector<uint8_t> space = {1, static_cast<uint8_t>(e.shape.size()), 0, 0, 0, 0, 0, 0};
                for (auto s : e.shape)
                {
                    for (int i = 0; i < 8; ++i)
                    {
                        space.push_back(static_cast<uint8_t>(s >> (8 * i)));
                    }
                }
                std::vector<uint8_t> type = e.kind == Kind::Interval ? interval_body() : type_body(e.kind);
                std::vector<uint8_t> fill = {2, 2, 2, 1, 0, 0, 0, 0}; // version 2: late allocation, default value
                std::vector<uint8_t> layout(18, 0);
                layout[0] = 3; // version 3
                layout[1] = 1; // contiguous
                for (int i = 0; i < 8; ++i)
                {
                    layout[2 + i]  = static_cast<uint8_t>(data >> (8 * i));
                    layout[10 + i] = static_cast<uint8_t>(static_cast<uint64_t>(e.bytes.size()) >> (8 * i));
                }
                return emit_header({{0x0001, space}, {0x0003, type}, {0x0005, fill}, {0x0008, layout}});
            }

            uint64_t emit_group(Group& g)
            {
                // members sorted by name: children first, then the group's own structures
                std::vector<std::pair<std::string, uint64_t>> members;
                std::map<std::string, Group*> subgroups;
                for (auto& kv : g.groups)
                {
                    members.push_back({kv.first, emit_group(*kv.second)});
                    subgroups[kv.first] = kv.second.get();
                }
                for (auto& kv : g.datasets)
                {
                    members.push_back({kv.first, emit_dataset(kv.second)});
                }
                std::sort(members.begin(), members.end(), [](const auto& a, const auto& b) { return std::strcmp(a.first.c_str(), b.first.c_str()) < 0; });
                // local heap: "" at offset 0, then the names, each padded to 8 bytes
                std::vector<uint64_t> name_off;
                uint64_t seg = 8;
                for (auto& m : members)
                {
                    name_off.push_back(seg);
                    seg += (m.first.size() + 1 + 7) & ~uint64_t(7);
                }
                const uint64_t heap = alloc(32);
                const uint64_t segd = alloc(seg);
                std::memcpy(&m_out[heap], "HEAP", 4);
                put64(heap + 8, seg);
                put64(heap + 16, UNDEF); // no free block
                put64(heap + 24, segd);
                for (size_t k = 0; k < members.size(); ++k)
                {
                    std::memcpy(&m_out[segd + name_off[k]], members[k].first.c_str(), members[k].first.size());
                }
                // symbol table nodes, 8 entries each, under one B-tree node of at most
                // 2 * 16 children
                const size_t per = 8, nsnod = std::max<size_t>(1, (members.size() + per - 1) / per);
                if (nsnod > 32)
                {
                    m_too_many = true;
                    return 0;
                }
                std::vector<uint64_t> snods;
                for (size_t s = 0; s < nsnod; ++s)
                {
                    const uint64_t at = alloc(8 + per * 40);
                    std::memcpy(&m_out[at], "SNOD", 4);
                    put8(at + 4, 1);
                    const size_t b = s * per, e = std::min(members.size(), b + per);
                    put16(at + 6, static_cast<uint16_t>(e - b));
                    for (size_t k = b; k < e; ++k)
                    {
                        const uint64_t q = at + 8 + (k - b) * 40;
                        put64(q, name_off[k]);
                        put64(q + 8, members[k].second);
                        auto it = subgroups.find(members[k].first);
                        if (it != subgroups.end())
                        {
                            put32(q + 16, 1);
                            put64(q + 24, it->second->btree);
                            put64(q + 32, it->second->heap);
                        }
                    }
                    snods.push_back(at);
                }
                // one B-tree node (level 0) over the symbol table nodes; full size for 2 * 16 children
                const uint64_t bt = alloc(24 + 33 * 8 + 32 * 8);
                std::memcpy(&m_out[bt], "TREE", 4);
                put8(bt + 4, 0);
                put8(bt + 5, 0);
                put16(bt + 6, static_cast<uint16_t>(members.empty() ? 0 : snods.size()));
                put64(bt + 8, UNDEF);
                put64(bt + 16, UNDEF);
                uint64_t p = bt + 24;
                put64(p, 0); // key 0: the empty name
                p += 8;
                for (size_t s = 0; s < snods.size() && !members.empty(); ++s)
                {
                    put64(p, snods[s]);
                    const size_t last = std::min(members.size(), (s + 1) * per) - 1;
                    put64(p + 8, name_off[last]);
                    p += 16;
                }
                g.btree = bt;
                g.heap  = heap;
                std::vector<uint8_t> stab(16);
                for (int i = 0; i < 8; ++i)
                {
                    stab[i]     = static_cast<uint8_t>(bt >> (8 * i));
                    stab[8 + i] = static_cast<uint8_t>(heap >> (8 * i));
                }
                return emit_header({{0x0011, stab}});
            }

            Group m_root;
            std::vector<uint8_t> m_out;
            bool m_too_many = false;
        };

        // --------------------------------------------------------------- reader
        struct Array
        {
            int cls      = -1;   // 0 fixed point, 1 floating point, 6 compound
            bool is_signed = false;
            size_t size  = 0;    // element size in bytes
            std::vector<uint64_t> shape;
            std::vector<uint8_t> bytes;
            std::map<std::string, size_t> members;     // compound member name -> byte offset
            std::map<std::string, size_t> member_size; // compound member name -> byte size

            uint64_t count() const
            {
                uint64_t n = 1;
                for (auto s : shape)
                {
                    n *= s;
                }
                return n;
            }

            // a compound member of `n` bytes lying inside the record
            bool member(const std::string& name, size_t n) const
            {
                auto o = members.find(name);
                auto z = member_size.find(name);
                return o != members.end() && z != member_size.end() && z->second == n && o->second <= size && n <= size - o->second;
            }
        };

        class Reader
        {
          public:

            bool open(const std::string& filename, std::string& err)
            {
                FILE* f = std::fopen(filename.c_str(), "rb");
                if (!f)
                {
                    err = "cannot open " + filename;
                    return false;
                }
                std::fseek(f, 0, SEEK_END);
                const long n = std::ftell(f);
                std::fseek(f, 0, SEEK_SET);
                m_b.resize(n > 0 ? static_cast<size_t>(n) : 0);
                const bool ok = n > 0 && std::fread(m_b.data(), 1, m_b.size(), f) == m_b.size();
                std::fclose(f);
                if (!ok || m_b.size() < 96 || std::memcmp(m_b.data(), "\x89HDF\r\n\x1a\n", 8) != 0)
                {
                    err = filename + " is not an HDF5 file";
                    return false;
                }
                if (m_b[8] != 0 || m_b[13] != 8 || m_b[14] != 8)
                {
                    err = filename + ": only superblock version 0 with 8-byte offsets and lengths is read";
                    return false;
                }
                m_root_header = u64(56 + 8); // root group symbol table entry: its object header
                m_name             = filename;
                return true;
            }

            // object header address of a path, UNDEF if absent
            uint64_t locate(const std::string& path, std::string& err) const
            {
                uint64_t obj = m_root_header;
                size_t p     = path.empty() || path[0] != '/' ? 0 : 1;
                while (p < path.size())
                {
                    size_t q = path.find('/', p);
                    if (q == std::string::npos)
                    {
                        q = path.size();
                    }
                    const std::string name = path.substr(p, q - p);
                    uint64_t btree = 0, heap = 0;
                    if (!symbol_table(obj, btree, heap, err))
                    {
                        return UNDEF;
                    }
                    int budget = 1 << 16;
                    obj        = lookup(btree, heap, name, err, 0, budget);
                    if (obj == UNDEF)
                    {
                        return UNDEF;
                    }
                    p = q + 1;
                }
                return obj;
            }

            bool exists(const std::string& path) const
            {
                std::string err;
                return locate(path, err) != UNDEF && err.empty();
            }

            bool read(const std::string& path, Array& out, std::string& err) const
            {
                const uint64_t obj = locate(path, err);
                if (obj == UNDEF)
                {
                    if (err.empty())
                    {
                        err = m_name + ": no dataset " + path;
                    }
                    return false;
                }
                std::vector<Msg> msgs;
                if (!messages(obj, msgs, err))
                {
                    return false;
                }
                bool have_space = false, have_type = false, have_layout = false;
                uint64_t addr = UNDEF, len = 0;
                for (auto& m : msgs)
                {
                    // every field read below lies inside the message's own m.size bytes
                    if (m.type == 0x0001)
                    {
                        // version 1: dims after 8 bytes; version 2: after 4 (a scalar has no dims)
                        const int ver = m.size >= 2 ? m_b[m.at] : 0, nd = m.size >= 2 ? m_b[m.at + 1] : 0;
                        const uint64_t p = m.at + (ver == 1 ? 8 : 4);
                        if ((ver != 1 && ver != 2) || nd > 32 || p + 8 * static_cast<uint64_t>(nd) > m.at + m.size)
                        {
                            err = m_name + ": " + path + ": malformed dataspace";
                            return false;
                        }
                        out.shape.clear();
                        for (int k = 0; k < nd; ++k)
                        {
                            out.shape.push_back(u64(p + 8 * k));
                        }
                        have_space = true;
                    }
                    else if (m.type == 0x0003)
                    {
                        if (!datatype(m.at, m.at + m.size, out, err))
                        {
                            return false;
                        }
                        have_type = true;
                    }
                    else if (m.type == 0x000B)
                    {
                        err = m_name + ": " + path + " is filtered (compressed), which is not read";
                        return false;
                    }
                    else if (m.type == 0x0008)
                    {
                        const int ver = m.size >= 4 ? m_b[m.at] : 0;
                        if (ver != 3)
                        {
                            err = m_name + ": " + path + ": layout message version " + std::to_string(ver) + " is not read";
                            return false;
                        }
                        const int cls = m_b[m.at + 1];
                        if (cls == 1 && m.size >= 18)
                        {
                            addr = u64(m.at + 2);
                            len  = u64(m.at + 10);
                        }
                        else if (cls == 0)
                        {
                            len  = static_cast<uint64_t>(m_b[m.at + 2]) | (static_cast<uint64_t>(m_b[m.at + 3]) << 8);
                            addr = m.at + 4;
                            if (len > m.size - 4u)
                            {
                                err = m_name + ": " + path + ": malformed compact layout";
                                return false;
                            }
                        }
                        else if (cls == 1)
                        {
                            err = m_name + ": " + path + ": malformed contiguous layout";
                            return false;
                        }
                        else
                        {
                            err = m_name + ": " + path + " is chunked, which is not read";
                            return false;
                        }
                        have_layout = true;
                    }
                }
                if (!have_space || !have_type || !have_layout)
                {
                    err = m_name + ": " + path + " is not a dataset";
                    return false;
                }
                // the element count and byte size, refused where they would overflow
                uint64_t nbytes = out.size;
                for (auto d : out.shape)
                {
                    if (d != 0 && nbytes > m_b.size() / d)
                    {
                        nbytes = UNDEF;
                        break;
                    }
                    nbytes *= d;
                }
                if (out.size == 0 && out.count() != 0)
                {
                    err = m_name + ": " + path + ": zero-sized elements";
                    return false;
                }
                if (nbytes == 0)
                {
                    out.bytes.clear();
                    return true;
                }
                if (len < nbytes || !in_file(addr, nbytes))
                {
                    err = m_name + ": " + path + ": data outside the file";
                    return false;
                }
                out.bytes.assign(m_b.begin() + static_cast<long>(addr), m_b.begin() + static_cast<long>(addr + nbytes));
                return true;
            }

          private:

            struct Msg
            {
                uint16_t type;
                uint64_t at;
                uint16_t size;
            };

            uint64_t u64(uint64_t at) const
            {
                uint64_t v = 0;
                for (int k = 7; k >= 0; --k)
                {
                    v = (v << 8) | m_b[at + k];
                }
                return v;
            }

            uint32_t u32(uint64_t at) const
            {
                return static_cast<uint32_t>(m_b[at]) | (static_cast<uint32_t>(m_b[at + 1]) << 8) | (static_cast<uint32_t>(m_b[at + 2]) << 16)
                     | (static_cast<uint32_t>(m_b[at + 3]) << 24);
            }

            uint16_t u16(uint64_t at) const
            {
                return static_cast<uint16_t>(m_b[at] | (m_b[at + 1] << 8));
            }

            bool in_file(uint64_t at, uint64_t n) const
            {
                return at != UNDEF && at <= m_b.size() && n <= m_b.size() - at;
            }

            bool messages(uint64_t obj, std::vector<Msg>& out, std::string& err) const
            {
                if (!in_file(obj, 16) || m_b[obj] != 1)
                {
                    err = m_name + ": only version 1 object headers are read";
                    return false;
                }
                const uint16_t nmsg = u16(obj + 2);
                std::vector<std::pair<uint64_t, uint64_t>> blocks = {{obj + 16, u32(obj + 8)}};
                for (size_t bi = 0; bi < blocks.size() && out.size() < nmsg; ++bi)
                {
                    uint64_t p         = blocks[bi].first;
                    const uint64_t end = p + blocks[bi].second;
                    if (!in_file(p, blocks[bi].second))
                    {
                        err = m_name + ": object header outside the file";
                        return false;
                    }
                    while (p + 8 <= end && out.size() < nmsg)
                    {
                        Msg m{u16(p), p + 8, u16(p + 2)};
                        if (m.at + m.size > end)
                        {
                            err = m_name + ": malformed object header";
                            return false;
                        }
                        if (m.type == 0x0010)
                        {
                            if (m.size < 16 || blocks.size() > 4096)
                            {
                                err = m_name + ": malformed object header continuation";
                                return false;
                            }
                            blocks.push_back({u64(m.at), u64(m.at + 8)});
                        }
                        out.push_back(m);
                        p = m.at + m.size;
                    }
                }
                return true;
            }

            bool symbol_table(uint64_t obj, uint64_t& btree, uint64_t& heap, std::string& err) const
            {
                std::vector<Msg> msgs;
                if (!messages(obj, msgs, err))
                {
                    return false;
                }
                for (auto& m : msgs)
                {
                    if (m.type == 0x0011 && m.size >= 16)
                    {
                        btree = u64(m.at);
                        heap  = u64(m.at + 8);
                        return true;
                    }
                }
                err = m_name + ": a path component is not a (symbol-table) group";
                return false;
            }

            std::string heap_name(uint64_t heap, uint64_t off) const
            {
                if (!in_file(heap, 32) || std::memcmp(&m_b[heap], "HEAP", 4) != 0)
                {
                    return std::string();
                }
                const uint64_t data = u64(heap + 24);
                const uint64_t size = u64(heap + 8);
                if (off >= size || !in_file(data, size))
                {
                    return std::string();
                }
                const char* s = reinterpret_cast<const char*>(&m_b[data + off]);
                return std::string(s, strnlen(s, static_cast<size_t>(size - off)));
            }

            // `budget` bounds the nodes visited, so that a B-tree whose children repeat ends quickly
            uint64_t lookup(uint64_t node, uint64_t heap, const std::string& name, std::string& err, int depth, int& budget) const
            {
                if (depth > 64 || --budget < 0 || !in_file(node, 24) || std::memcmp(&m_b[node], "TREE", 4) != 0 || m_b[node + 4] != 0)
                {
                    err = m_name + ": malformed group B-tree";
                    return UNDEF;
                }
                const int level  = m_b[node + 5];
                const int used   = u16(node + 6);
                uint64_t p       = node + 24 + 8; // after key 0
                for (int k = 0; k < used; ++k, p += 16)
                {
                    if (!in_file(p, 16))
                    {
                        err = m_name + ": malformed group B-tree";
                        return UNDEF;
                    }
                    const uint64_t child = u64(p);
                    if (level > 0)
                    {
                        const uint64_t r = lookup(child, heap, name, err, depth + 1, budget);
                        if (r != UNDEF || !err.empty())
                        {
                            return r;
                        }
                        continue;
                    }
                    if (!in_file(child, 8) || std::memcmp(&m_b[child], "SNOD", 4) != 0)
                    {
                        err = m_name + ": malformed symbol table node";
                        return UNDEF;
                    }
                    const int nsym = u16(child + 6);
                    for (int s = 0; s < nsym; ++s)
                    {
                        const uint64_t q = child + 8 + 40 * static_cast<uint64_t>(s);
                        if (!in_file(q, 40))
                        {
                            err = m_name + ": malformed symbol table node";
                            return UNDEF;
                        }
                        if (heap_name(heap, u64(q)) == name)
                        {
                            return u64(q + 8);
                        }
                    }
                }
                return UNDEF;
            }

            // a datatype message at [at, lim)
            bool datatype(uint64_t at, uint64_t lim, Array& out, std::string& err) const
            {
                if (at + 8 > lim)
                {
                    err = m_name + ": malformed datatype";
                    return false;
                }
                const int cls = m_b[at] & 0x0F, ver = m_b[at] >> 4;
                out.cls       = cls;
                out.size      = u32(at + 4);
                if (cls == 0)
                {
                    out.is_signed = (m_b[at + 1] & 0x08) != 0;
                    if (m_b[at + 1] & 0x01)
                    {
                        err = m_name + ": big-endian integers are not read";
                        return false;
                    }
                    return true;
                }
                if (cls == 1)
                {
                    if ((m_b[at + 1] & 0x41) != 0 || out.size != 8)
                    {
                        err = m_name + ": only little-endian binary64 floating point is read";
                        return false;
                    }
                    return true;
                }
                if (cls == 6)
                {
                    const int nm = u16(at + 1);
                    uint64_t p   = at + 8;
                    for (int m = 0; m < nm; ++m)
                    {
                        if (p >= lim)
                        {
                            err = m_name + ": malformed compound datatype";
                            return false;
                        }
                        const char* s   = reinterpret_cast<const char*>(&m_b[p]);
                        const size_t ln = strnlen(s, static_cast<size_t>(std::min<uint64_t>(lim - p, 256)));
                        std::string mname(s, ln);
                        size_t off = 0;
                        if (ver == 3)
                        {
                            p += ln + 1;
                            const int nb = out.size < 256 ? 1 : out.size < 65536 ? 2 : out.size < (1u << 24) ? 3 : 4;
                            if (p + nb > lim)
                            {
                                err = m_name + ": malformed compound datatype";
                                return false;
                            }
                            for (int k = 0; k < nb; ++k)
                            {
                                off |= static_cast<size_t>(m_b[p + k]) << (8 * k);
                            }
                            p += nb;
                        }
                        else
                        {
                            p += (ln + 1 + 7) & ~size_t(7);
                            if (p + 4 > lim)
                            {
                                err = m_name + ": malformed compound datatype";
                                return false;
                            }
                            off = u32(p);
                            p += ver == 1 ? 4 + 1 + 3 + 4 + 4 + 16 : 4;
                        }
                        // the member's own datatype message (fixed-point and floating-point members only)
                        if (p + 8 > lim)
                        {
                            err = m_name + ": malformed compound datatype";
                            return false;
                        }
                        const int mcls     = m_b[p] & 0x0F;
                        const size_t msize = u32(p + 4);
                        if (mcls != 0 && mcls != 1)
                        {
                            err = m_name + ": nested compound members are not read";
                            return false;
                        }
                        p += mcls == 0 ? 8 + 4 : 8 + 12;
                        if (p > lim || off > out.size || msize > out.size - off)
                        {
                            err = m_name + ": malformed compound datatype";
                            return false;
                        }
                        out.members[mname]     = off;
                        out.member_size[mname] = msize;
                    }
                    return true;
                }
                err = m_name + ": datatype class " + std::to_string(cls) + " is not read";
                return false;
            }

            std::vector<uint8_t> m_b;
            uint64_t m_root_header = 0;
            std::string m_name;
        };
    } // namespace h5
} // namespace sg
