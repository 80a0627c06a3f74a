// samurai's output and restart files for this path, through the minimal
// HDF5 layer of sg_h5.hpp (no libhdf5):
//  - save (io/hdf5.hpp:682-937, 1331-1336): <path>/<name>.h5 with
//    /mesh/points, /mesh/connectivity and /mesh/fields/<field>, plus the
//    XDMF description <path>/<name>.xdmf;
//  - dump / load (io/restart.hpp:50-201, 236-463): the CellArray of the leaf
//    cells level by level (LevelCellArray intervals and offsets, as
//    level_cell_array.hpp:1005-1077 lays them out) and each field's leaf
//    values in for_each_cell order.
// Host code: the mesh and the fields are read or written through the C ABI
// of the library (leaf cells, interval lists, field downloads and uploads).
#include <algorithm>
#include <cinttypes>
#include <cstdio>
#include <cstring>
#include <new>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/samurai_gpu.h"
#include "sg_ctx.cuh"
#include "sg_csr.hpp"
#include "sg_h5.hpp"

#include "sg_handles.cuh"


// an ordered list of scalar and vector fields for save / dump / load
struct sg_io_s
{
    struct Item
    {
        sg_field_t f  = nullptr;
        sg_vfield_t v = nullptr;
    };
    std::vector<Item> items;
};

namespace
{
    int iofail(int code, const std::string& msg)
    {
        sg::set_last_error(msg.c_str(), nullptr);
        return code;
    }

    std::string file_of(const char* path, const char* filename, const char* ext)
    {
        std::string p = path ? path : "";
        if (!p.empty() && p.back() != '/')
        {
            p += '/';
        }
        return p + filename + ext;
    }

    struct Leaves
    {
        int dim = 2;
        std::vector<int> level, coords;
        std::vector<long long> index;
        long long n = 0, nb_ref = 0;
    };

    int leaves(sg_mesh_t mesh, Leaves& L)
    {
        L.dim = mesh->ctx.g.dim;
        if (int st = sg_mesh_counts(mesh, &L.n, &L.nb_ref))
        {
            return st;
        }
        L.level.resize(static_cast<size_t>(L.n));
        L.coords.resize(static_cast<size_t>(L.n) * L.dim);
        L.index.resize(static_cast<size_t>(L.n));
        if (L.n == 0)
        {
            return SG_OK;
        }
        return sg_mesh_get_cells(mesh, L.level.data(), L.coords.data(), L.index.data(), L.n);
    }

    // leaf values of one scalar field, for_each_cell order
    int leaf_values(sg_field_t f, const Leaves& L, std::vector<double>& out)
    {
        std::vector<double> full(static_cast<size_t>(L.nb_ref));
        if (int st = sg_field_download(f, full.data(), L.nb_ref))
        {
            return st;
        }
        out.resize(static_cast<size_t>(L.n));
        for (long long k = 0; k < L.n; ++k)
        {
            out[static_cast<size_t>(k)] = full[static_cast<size_t>(L.index[static_cast<size_t>(k)])];
        }
        return SG_OK;
    }

    const char* element_name(int dim)
    {
        return dim == 2 ? "Quadrilateral" : "Hexahedron"; // io/hdf5.hpp:44-58
    }

    // dump(file, name, data) (io/restart.hpp:52-88): <name>/partition = {0, n} and <name>/data
    template <class T>
    void dump_vector(sg::h5::Writer& w, const std::string& name, sg::h5::Kind kind, const std::vector<T>& data)
    {
        if (data.empty())
        {
            return;
        }
        const uint64_t part[2] = {0, static_cast<uint64_t>(data.size())};
        w.add(name + "/partition", sg::h5::Kind::U64, {2}, part);
        w.add(name + "/data", kind, {static_cast<uint64_t>(data.size())}, data.data());
    }

    int check_io(sg_mesh_t mesh, sg_io_t io, const char* what)
    {
        if (!io)
        {
            return SG_OK;
        }
        for (auto& it : io->items)
        {
            if ((it.f && it.f->mesh != mesh) || (it.v && it.v->mesh != mesh))
            {
                return iofail(SG_ERR_ARG, std::string(what) + ": every field must live on the mesh");
            }
        }
        return SG_OK;
    }
} // namespace

extern "C"
{
    int sg_io_create(sg_io_t* out)
    try
    {
        if (!out)
        {
            return iofail(SG_ERR_ARG, "sg_io_create: null output");
        }
        *out = new (std::nothrow) sg_io_s();
        return *out ? SG_OK : iofail(SG_ERR_CAPACITY, "sg_io_create: out of host memory");
    }
    SG_API_CATCH(sg_io_create)

    int sg_io_destroy(sg_io_t io)
    try
    {
        delete io;
        return SG_OK;
    }
    SG_API_CATCH(sg_io_destroy)

    int sg_io_add_field(sg_io_t io, sg_field_t f)
    try
    {
        if (!io || !f)
        {
            return iofail(SG_ERR_ARG, "sg_io_add_field: null argument");
        }
        io->items.push_back({f, nullptr});
        return SG_OK;
    }
    SG_API_CATCH(sg_io_add_field)

    int sg_io_add_vector_field(sg_io_t io, sg_vfield_t v)
    try
    {
        if (!io || !v)
        {
            return iofail(SG_ERR_ARG, "sg_io_add_vector_field: null argument");
        }
        io->items.push_back({nullptr, v});
        return SG_OK;
    }
    SG_API_CATCH(sg_io_add_vector_field)

    static int save_body(const char* path, const char* filename, sg_mesh_t mesh, sg_io_t fields)
    {
        if (!filename || !*filename || !mesh)
        {
            return iofail(SG_ERR_ARG, "sg_save: need a file name and a mesh");
        }
        if (int st = check_io(mesh, fields, "sg_save"))
        {
            return st;
        }
        Leaves L;
        if (int st = leaves(mesh, L))
        {
            return st;
        }
        const int D         = L.dim;
        const int corners   = 1 << D;
        const int max_level = mesh->ctx.cfg.max_level;
        sg::h5::Writer w;
        std::string grid;
        if (L.n > 0)
        {
            // points and connectivity (io/hdf5.hpp:85-144): corner ids in order of first appearance
            static const int e2[4][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}};
            static const int e3[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
            const uint64_t span = (uint64_t(1) << max_level) + 1;
            std::unordered_map<uint64_t, uint64_t> ids;
            ids.reserve(static_cast<size_t>(L.n) * 2);
            std::vector<uint64_t> conn(static_cast<size_t>(L.n) * corners);
            std::vector<double> pts;
            pts.reserve(static_cast<size_t>(L.n) * 3 * 2);
            const double fine = 1.0 / static_cast<double>(uint64_t(1) << max_level);
            for (long long k = 0; k < L.n; ++k)
            {
                const int sh = max_level - L.level[static_cast<size_t>(k)];
                for (int c = 0; c < corners; ++c)
                {
                    const int* e = D == 2 ? e2[c] : e3[c];
                    uint64_t X[3] = {0, 0, 0};
                    uint64_t key  = 0;
                    for (int d = D - 1; d >= 0; --d)
                    {
                        X[d] = static_cast<uint64_t>(L.coords[static_cast<size_t>(k) * D + d] + e[d]) << sh;
                        key  = key * span + X[d];
                    }
                    auto ins = ids.emplace(key, static_cast<uint64_t>(ids.size()));
                    if (ins.second)
                    {
                        for (int d = 0; d < 3; ++d)
                        {
                            // exact: dyadic coordinates of the unit box
                            pts.push_back(d < D ? static_cast<double>(X[d]) * fine : 0.);
                        }
                    }
                    conn[static_cast<size_t>(k) * corners + c] = ins.first->second;
                }
            }
            const uint64_t npts = ids.size();
            w.add("/mesh/connectivity", sg::h5::Kind::U64, {static_cast<uint64_t>(L.n), static_cast<uint64_t>(corners)}, conn.data());
            w.add("/mesh/points", sg::h5::Kind::F64, {npts, 3}, pts.data());
            const std::string h5name = std::string(filename) + ".h5";
            char buf[512];
            grid += "        <Grid Name=\"mesh\">\n";
            std::snprintf(buf, sizeof(buf), "            <Topology TopologyType=\"%s\" NumberOfElements=\"%lld\">\n", element_name(D), L.n);
            grid += buf;
            std::snprintf(buf, sizeof(buf), "                <DataItem Dimensions=\"%lld\" Format=\"HDF\">", L.n * corners);
            grid += buf + h5name + ":/mesh/connectivity</DataItem>\n";
            grid += "            </Topology>\n";
            grid += "            <Geometry GeometryType=\"XYZ\">\n";
            std::snprintf(buf, sizeof(buf), "                <DataItem Dimensions=\"%" PRIu64 "\" Format=\"HDF\">", npts * 3);
            grid += buf + h5name + ":/mesh/points</DataItem>\n";
            grid += "            </Geometry>\n";
            // fields (io/hdf5.hpp:839-897): one dataset per component, <name>_<c> for vector fields
            std::vector<std::pair<std::string, sg_field_t>> comps;
            if (fields)
            {
                for (auto& it : fields->items)
                {
                    if (it.f)
                    {
                        comps.push_back({it.f->f.name, it.f});
                    }
                    else
                    {
                        for (size_t c = 0; c < it.v->comp.size(); ++c)
                        {
                            comps.push_back({it.v->name + "_" + std::to_string(c), it.v->comp[c]});
                        }
                    }
                }
            }
            std::vector<double> vals;
            for (auto& fc : comps)
            {
                if (int st = leaf_values(fc.second, L, vals))
                {
                    return st;
                }
                const std::string dpath = "/mesh/fields/" + fc.first;
                w.add(dpath, sg::h5::Kind::F64, {static_cast<uint64_t>(L.n)}, vals.data());
                grid += "            <Attribute Name=\"" + fc.first + "\" Center=\"Cell\">\n";
                std::snprintf(buf, sizeof(buf), "                <DataItem Dimensions=\"%lld\" Format=\"HDF\" Precision=\"8\">", L.n);
                grid += buf + h5name + ":" + dpath + "</DataItem>\n";
                grid += "            </Attribute>\n";
            }
            grid += "        </Grid>\n";
        }
        std::string err;
        if (!w.save(file_of(path, filename, ".h5"), err))
        {
            return iofail(SG_ERR_ARG, "sg_save: " + err);
        }
        std::string xdmf = "<?xml version=\"1.0\"?>\n<Xdmf>\n";
        xdmf += grid.empty() ? "    <Domain />\n" : "    <Domain>\n" + grid + "    </Domain>\n";
        xdmf += "</Xdmf>\n";
        const std::string xname = file_of(path, filename, ".xdmf");
        FILE* f                 = std::fopen(xname.c_str(), "wb");
        if (!f || std::fwrite(xdmf.data(), 1, xdmf.size(), f) != xdmf.size())
        {
            if (f)
            {
                std::fclose(f);
            }
            return iofail(SG_ERR_ARG, "sg_save: cannot write " + xname);
        }
        std::fclose(f);
        return SG_OK;
    }

    static int dump_body(const char* path, const char* filename, sg_mesh_t mesh, sg_io_t fields)
    {
        if (!filename || !*filename || !mesh)
        {
            return iofail(SG_ERR_ARG, "sg_dump: need a file name and a mesh");
        }
        if (int st = check_io(mesh, fields, "sg_dump"))
        {
            return st;
        }
        sg::Ctx& c  = mesh->ctx;
        const int D = c.g.dim;
        sg::h5::Writer w;
        const uint64_t one = 1, dim = static_cast<uint64_t>(D);
        const uint64_t minl = static_cast<uint64_t>(c.cfg.min_level), maxl = static_cast<uint64_t>(c.cfg.max_level);
        const double origin[3] = {0., 0., 0.}, scaling = 1.;
        w.add("/n_process", sg::h5::Kind::U64, {}, &one);
        w.add("/mesh/dim", sg::h5::Kind::U64, {}, &dim);
        w.add("/mesh/min_level", sg::h5::Kind::U64, {}, &minl);
        w.add("/mesh/max_level", sg::h5::Kind::U64, {}, &maxl);
        w.add("/mesh/origin_point", sg::h5::Kind::F64, {dim}, origin);
        w.add("/mesh/scaling_factor", sg::h5::Kind::F64, {}, &scaling);
        // the leaf CellArray, level by level (io/restart.hpp:90-155)
        for (int l = 0; l <= c.cfg.max_level; ++l)
        {
            long long ni = 0;
            if (int st = sg_mesh_count_intervals(mesh, SG_CELLS, l, &ni))
            {
                return st;
            }
            if (ni == 0)
            {
                continue;
            }
            std::vector<long long> rows(static_cast<size_t>(ni) * (D + 2));
            if (int st = sg_mesh_get_intervals(mesh, SG_CELLS, l, rows.data(), ni))
            {
                return st;
            }
            sg::csr::LevelCSR csr;
            sg::csr::build_csr(D, rows, csr);
            const std::string base = "/mesh/level/" + std::to_string(l) + "/dim/";
            for (int d = 0; d < D; ++d)
            {
                dump_vector(w, base + std::to_string(d) + "/intervals", sg::h5::Kind::Interval, csr.iv[d]);
            }
            for (int d = 1; d < D; ++d)
            {
                dump_vector(w, base + std::to_string(d) + "/offsets", sg::h5::Kind::U64, csr.off[d - 1]);
            }
        }
        // fields (io/restart.hpp:157-174): n_comp and the leaf values, components side by side
        if (fields)
        {
            Leaves L;
            if (int st = leaves(mesh, L))
            {
                return st;
            }
            std::vector<double> vals;
            for (auto& it : fields->items)
            {
                const std::string name = it.f ? it.f->f.name : it.v->name;
                const uint64_t nc      = it.f ? 1 : it.v->comp.size();
                std::vector<double> data(static_cast<size_t>(L.n) * nc);
                for (uint64_t cc = 0; cc < nc; ++cc)
                {
                    if (int st = leaf_values(it.f ? it.f : it.v->comp[cc], L, vals))
                    {
                        return st;
                    }
                    for (long long k = 0; k < L.n; ++k)
                    {
                        data[static_cast<size_t>(k) * nc + cc] = vals[static_cast<size_t>(k)];
                    }
                }
                w.add("/fields/" + name + "/n_comp", sg::h5::Kind::U64, {}, &nc);
                dump_vector(w, "/fields/" + name + "/data", sg::h5::Kind::F64, data);
            }
        }
        std::string err;
        if (!w.save(file_of(path, filename, ".h5"), err))
        {
            return iofail(SG_ERR_ARG, "sg_dump: " + err);
        }
        return SG_OK;
    }

    static int restart_levels_body(const char* path, const char* filename, int* dim, int* min_level, int* max_level)
    {
        if (!filename || !dim || !min_level || !max_level)
        {
            return iofail(SG_ERR_ARG, "sg_restart_levels: null argument");
        }
        sg::h5::Reader r;
        std::string err;
        sg::h5::Array a;
        if (!r.open(file_of(path, filename, ".h5"), err))
        {
            return iofail(SG_ERR_NOTFOUND, "sg_restart_levels: " + err);
        }
        int* outs[3]          = {dim, min_level, max_level};
        const char* names[3]  = {"/mesh/dim", "/mesh/min_level", "/mesh/max_level"};
        for (int k = 0; k < 3; ++k)
        {
            if (!r.read(names[k], a, err) || a.cls != 0 || a.size != 8 || a.count() != 1)
            {
                return iofail(SG_ERR_ARG, "sg_restart_levels: " + (err.empty() ? std::string(names[k]) + " is not an integer" : err));
            }
            uint64_t v;
            std::memcpy(&v, a.bytes.data(), 8);
            *outs[k] = static_cast<int>(v);
        }
        return SG_OK;
    }

    static int load_body(const char* path, const char* filename, sg_mesh_t mesh, sg_io_t fields)
    {
        if (!filename || !mesh)
        {
            return iofail(SG_ERR_ARG, "sg_load: need a file name and a mesh");
        }
        if (int st = check_io(mesh, fields, "sg_load"))
        {
            return st;
        }
        sg::Ctx& c  = mesh->ctx;
        const int D = c.g.dim;
        sg::h5::Reader r;
        std::string err;
        const std::string fname = file_of(path, filename, ".h5");
        if (!r.open(fname, err))
        {
            return iofail(SG_ERR_NOTFOUND, "sg_load: " + err);
        }
        auto read_u64 = [&](const std::string& p, std::vector<uint64_t>& out) -> bool
        {
            sg::h5::Array a;
            if (!r.read(p, a, err))
            {
                return false;
            }
            if (a.cls != 0 || a.size != 8)
            {
                err = fname + ": " + p + " is not a 64-bit integer array";
                return false;
            }
            out.resize(static_cast<size_t>(a.count()));
            std::memcpy(out.data(), a.bytes.data(), a.bytes.size());
            return true;
        };
        std::vector<uint64_t> v;
        if (!read_u64("/n_process", v) || v.size() != 1 || v[0] != 1)
        {
            return iofail(SG_ERR_ARG, "sg_load: " + (err.empty() ? std::string("the file was written by more than one process") : err));
        }
        int fd = 0, fmin = 0, fmax = 0;
        if (int st = sg_restart_levels(path, filename, &fd, &fmin, &fmax))
        {
            return st;
        }
        if (fd != D || fmin != c.cfg.min_level || fmax != c.cfg.max_level)
        {
            return iofail(SG_ERR_ARG, "sg_load: the file's dimension and levels (" + std::to_string(fd) + ", " + std::to_string(fmin) + ", "
                                          + std::to_string(fmax) + ") differ from the mesh's; create the mesh with sg_restart_levels");
        }
        // leaf cells, for_each_cell order (io/restart.hpp:288-321, level_cell_array.hpp:1005-1077).  The leaves
        // of a mesh tile the box, so their volume, counted in cells of the finest level, is at most the box's:
        // each level may decode at most the cells that the volume left over by the coarser levels still holds
        // (and the library holds fewer than 2^31 cells)
        std::vector<int> lv, co;
        const int vbits     = D * fmax; // at most 3 * 21 bits (sg_mesh_create's level limits)
        uint64_t vol_left   = (vbits >= 64) ? ~uint64_t(0) : (uint64_t(1) << vbits);
        for (int l = fmin; l <= fmax; ++l)
        {
            const std::string base = "/mesh/level/" + std::to_string(l) + "/dim/";
            if (!r.exists("/mesh/level/" + std::to_string(l)))
            {
                continue;
            }
            sg::csr::LevelCSR csr;
            for (int d = 0; d < D; ++d)
            {
                sg::h5::Array a;
                const std::string p = base + std::to_string(d) + "/intervals";
                if (!r.read(p + "/data", a, err) || a.cls != 6 || a.size != 24 || !a.member("start", 4) || !a.member("end", 4)
                    || !a.member("index", 8))
                {
                    return iofail(SG_ERR_ARG, "sg_load: " + (err.empty() ? p + " is not an Interval array" : err));
                }
                auto& iv = csr.iv[d];
                iv.resize(static_cast<size_t>(a.count()));
                for (size_t k = 0; k < iv.size(); ++k)
                {
                    const uint8_t* q = a.bytes.data() + 24 * k;
                    std::memcpy(&iv[k].start, q + a.members.at("start"), 4);
                    std::memcpy(&iv[k].end, q + a.members.at("end"), 4);
                    std::memcpy(&iv[k].index, q + a.members.at("index"), 8);
                }
            }
            for (int d = 1; d < D; ++d)
            {
                if (!read_u64(base + std::to_string(d) + "/offsets/data", csr.off[d - 1]))
                {
                    return iofail(SG_ERR_ARG, "sg_load: " + err);
                }
            }
            const size_t before    = co.size();
            const int shift        = D * (fmax - l); // finest cells per cell of level l: 2^shift
            uint64_t budget        = vol_left >> shift;
            const uint64_t cap     = (uint64_t(1) << 31) - 1 - lv.size();
            budget                 = budget < cap ? budget : cap;
            const sg::csr::Decode dec = sg::csr::decode_csr(D, l, csr, co, budget);
            if (dec == sg::csr::Decode::outside)
            {
                return iofail(SG_ERR_ARG, "sg_load: " + fname + ": interval outside the level-" + std::to_string(l) + " box");
            }
            if (dec != sg::csr::Decode::ok)
            {
                return iofail(SG_ERR_ARG, "sg_load: " + fname + ": inconsistent intervals and offsets at level " + std::to_string(l));
            }
            const size_t got = (co.size() - before) / static_cast<size_t>(D);
            vol_left -= static_cast<uint64_t>(got) << shift; // got <= budget <= vol_left >> shift
            lv.insert(lv.end(), got, l);
        }
        {
            // the leaves tile the box: their volume is the box's, and no leaf lies inside a coarser one
            if (vol_left != 0)
            {
                return iofail(SG_ERR_ARG, "sg_load: " + fname + ": the file's leaf cells do not cover the box");
            }
            std::vector<std::vector<uint64_t>> keys(static_cast<size_t>(fmax + 1));
            auto key = [&](int x, int y, int z) { return (uint64_t(uint32_t(z)) << 42) | (uint64_t(uint32_t(y)) << 21) | uint64_t(uint32_t(x)); };
            for (size_t i = 0; i < lv.size(); ++i)
            {
                keys[static_cast<size_t>(lv[i])].push_back(key(co[D * i], co[D * i + 1], D == 3 ? co[D * i + 2] : 0));
            }
            for (auto& k : keys)
            {
                std::sort(k.begin(), k.end());
            }
            for (size_t i = 0; i < lv.size(); ++i)
            {
                for (int l = fmin; l < lv[i]; ++l)
                {
                    const int s = lv[i] - l;
                    const uint64_t a = key(co[D * i] >> s, co[D * i + 1] >> s, D == 3 ? co[D * i + 2] >> s : 0);
                    if (std::binary_search(keys[static_cast<size_t>(l)].begin(), keys[static_cast<size_t>(l)].end(), a))
                    {
                        return iofail(SG_ERR_ARG, "sg_load: " + fname + ": a leaf cell of level " + std::to_string(lv[i])
                                                      + " lies inside a leaf of level " + std::to_string(l));
                    }
                }
            }
        }
        if (int st = sg_mesh_set_cells(mesh, static_cast<long long>(lv.size()), lv.data(), co.data()))
        {
            return st;
        }
        {
            // samurai's restart holds exactly the file's leaves: cells repeated in the file, or overlapping
            // across levels, would merge into fewer cells, and the file's values would then belong to other cells
            long long nc = 0, nr = 0;
            if (int st = sg_mesh_counts(mesh, &nc, &nr))
            {
                return st;
            }
            if (nc != static_cast<long long>(lv.size()))
            {
                return iofail(SG_ERR_ARG, "sg_load: " + fname + ": the file's leaf cells repeat or overlap (" + std::to_string(lv.size())
                                              + " cells read, " + std::to_string(nc) + " distinct leaves)");
            }
        }
        // fields (io/restart.hpp:323-372): leaf values in for_each_cell order of the cells read
        if (fields)
        {
            long long nc = 0, nr = 0;
            if (int st = sg_mesh_counts(mesh, &nc, &nr))
            {
                return st;
            }
            for (auto& it : fields->items)
            {
                const std::string name = it.f ? it.f->f.name : it.v->name;
                const uint64_t ncomp   = it.f ? 1 : it.v->comp.size();
                if (name.empty())
                {
                    return iofail(SG_ERR_ARG, "sg_load: the field has no name");
                }
                std::vector<uint64_t> n_comp;
                if (!r.exists("/fields/" + name) || !read_u64("/fields/" + name + "/n_comp", n_comp) || n_comp.size() != 1)
                {
                    return iofail(SG_ERR_ARG, "sg_load: the field " + name + " does not exist in the file");
                }
                if (n_comp[0] != ncomp)
                {
                    return iofail(SG_ERR_ARG, "sg_load: the number of components of the field " + name + " does not match");
                }
                std::vector<double> data;
                if (nc > 0)
                {
                    sg::h5::Array a;
                    if (!r.read("/fields/" + name + "/data/data", a, err) || a.cls != 1
                        || a.count() != static_cast<uint64_t>(nc) * ncomp)
                    {
                        return iofail(SG_ERR_ARG, "sg_load: " + (err.empty() ? "the data of " + name + " does not match the mesh" : err));
                    }
                    data.resize(static_cast<size_t>(a.count()));
                    std::memcpy(data.data(), a.bytes.data(), a.bytes.size());
                }
                if (it.f)
                {
                    if (int st = sg_field_set_cells(it.f, data.data(), nc))
                    {
                        return st;
                    }
                }
                else if (int st = sg_vector_field_set_cells(it.v, data.data(), nc * static_cast<long long>(ncomp)))
                {
                    return st;
                }
            }
        }
        return SG_OK;
    }

    int sg_save(const char* path, const char* filename, sg_mesh_t mesh, sg_io_t fields)
    try
    {
        return save_body(path, filename, mesh, fields);
    }
    SG_API_CATCH(sg_save)

    int sg_dump(const char* path, const char* filename, sg_mesh_t mesh, sg_io_t fields)
    try
    {
        return dump_body(path, filename, mesh, fields);
    }
    SG_API_CATCH(sg_dump)

    int sg_restart_levels(const char* path, const char* filename, int* dim, int* min_level, int* max_level)
    try
    {
        return restart_levels_body(path, filename, dim, min_level, max_level);
    }
    SG_API_CATCH(sg_restart_levels)

    int sg_load(const char* path, const char* filename, sg_mesh_t mesh, sg_io_t fields)
    try
    {
        return load_body(path, filename, mesh, fields);
    }
    SG_API_CATCH(sg_load)
}
