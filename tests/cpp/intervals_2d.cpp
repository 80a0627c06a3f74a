// for_each_interval and u(level, i, j) through the drop-in header: after the
// advection demo's initial adaptation, prints for every leaf interval
// "level start end j index" and, for every leaf cell, "level i j u(level, i, j)",
// and checks that u(level, i, j) and u[cell] agree.  Usage: intervals_2d <out.txt>
#include <cstdio>
#include <string>

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
        auto config = samurai::mesh_config<dim>().min_level(3).max_level(7).max_stencil_size(2).disable_minimal_ghost_width();
        auto mesh   = samurai::mra::make_mesh(box, config);
        auto u      = samurai::make_scalar_field<double>("u", mesh);
        samurai::for_each_cell(mesh,
                               [&](auto& cell)
                               {
                                   auto c  = cell.center();
                                   u[cell] = ((c[0] - 0.4) * (c[0] - 0.4) + (c[1] - 0.6) * (c[1] - 0.6) < 0.04) ? 1. : 0.;
                               });
        samurai::make_bc<samurai::Dirichlet<1>>(u, 0.);
        auto MRadaptation = samurai::make_MRAdapt(u);
        MRadaptation(samurai::mra_config().epsilon(1e-3));
        FILE* f = std::fopen(argv[1], "w");
        if (!f)
        {
            return 1;
        }
        std::size_t mismatch = 0;
        samurai::for_each_interval(mesh,
                                   [&](std::size_t level, const auto& i, const auto& index)
                                   {
                                       std::fprintf(f, "I %zu %d %d %d %lld\n", level, i.start, i.end, index[0], i.index);
                                       for (int x = i.start; x < i.end; ++x)
                                       {
                                           std::fprintf(f, "C %zu %d %d %.17g\n", level, x, index[0], u(level, x, index[0]));
                                       }
                                   });
        samurai::for_each_cell(mesh,
                               [&](auto& cell)
                               {
                                   mismatch += (u(cell.level, cell.indices[0], cell.indices[1]) != u[cell]) ? 1 : 0;
                               });
        std::fclose(f);
        if (mismatch)
        {
            std::fprintf(stderr, "%zu cells disagree\n", mismatch);
            return 1;
        }
        return 0;
    }
    catch (const std::exception& e)
    {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
}
