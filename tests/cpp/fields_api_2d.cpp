// Field and mesh-id calls of the drop-in header: make_scalar_field with an
// initial value and with a function of the cell centre, u.fill, mesh.nb_cells
// per mesh id, and for_each_cell / for_each_interval over mesh[mesh_id].
// Prints "key value" lines.  Usage: fields_api_2d <out.txt>
#include <cstdio>

#include <samurai_gb300/samurai.hpp>

int main(int argc, char** argv)
{
    if (argc < 2)
    {
        return 2;
    }
    try
    {
        constexpr std::size_t dim = 2;
        const samurai::Box<double, dim> box({0., 0.}, {1., 1.});
        auto config    = samurai::mesh_config<dim>().min_level(2).max_level(6).max_stencil_size(2).disable_minimal_ghost_width();
        auto mesh      = samurai::mra::make_mesh(box, config);
        using mesh_id_t = typename decltype(mesh)::mesh_id_t;
        auto u = samurai::make_scalar_field<double>("u", mesh,
                                                    [](const auto& coords)
                                                    {
                                                        const double x = coords(0), y = coords(1);
                                                        return (x >= 0.3 && x <= 0.6 && y >= 0.4 && y <= 0.7) ? 1. : 0.;
                                                    });
        samurai::make_bc<samurai::Dirichlet<1>>(u, 0.);
        auto MRadaptation = samurai::make_MRAdapt(u);
        MRadaptation(samurai::mra_config().epsilon(1e-3));
        auto v = samurai::make_scalar_field<double>("v", mesh, 2.5);
        FILE* f = std::fopen(argv[1], "w");
        if (!f)
        {
            return 1;
        }
        std::fprintf(f, "cells %zu\n", mesh.nb_cells(mesh_id_t::cells));
        std::fprintf(f, "reference %zu\n", mesh.nb_cells(mesh_id_t::reference));
        std::fprintf(f, "cells_and_ghosts %zu\n", mesh.nb_cells(mesh_id_t::cells_and_ghosts));
        std::fprintf(f, "proj_cells %zu\n", mesh.nb_cells(mesh_id_t::proj_cells));
        std::fprintf(f, "union_cells %zu\n", mesh.nb_cells(mesh_id_t::union_cells));
        double su = 0., sv = 0.;
        std::size_t nref = 0;
        samurai::for_each_cell(mesh[mesh_id_t::cells], [&](const auto& cell) { su += u[cell]; sv += v[cell]; });
        samurai::for_each_cell(mesh[mesh_id_t::reference], [&](const auto&) { ++nref; });
        std::size_t nproj = 0;
        samurai::for_each_interval(mesh[mesh_id_t::proj_cells], [&](std::size_t, const auto& i, const auto&) { nproj += i.size(); });
        std::fprintf(f, "sum_u %.17g\nsum_v %.17g\nnref_walk %zu\nnproj_walk %zu\n", su, sv, nref, nproj);
        u.fill(-1.);
        double sf = 0.;
        samurai::for_each_cell(mesh, [&](const auto& cell) { sf += u[cell]; });
        std::fprintf(f, "sum_fill %.17g\n", sf);
        std::fclose(f);
        return 0;
    }
    catch (const std::exception& e)
    {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
}
