// A two-component advection in the style of samurai's demos, written against
// the GB300 drop-in header: make_vector_field<double, 2>, make_bc with one
// constant per component, make_MRAdapt on the vector field (its two details
// decide the mesh together), update_ghost_mr and unp1 = u - dt * upwind(a, u)
// on the vector field.  Usage:
//   vector_advection_2d <out.txt> [relative]
// Prints the number of steps, then "level i j u0 u1" for every leaf cell.
#include <cstdio>
#include <cstdlib>
#include <string>

#include <samurai_gb300/samurai.hpp>

template <class Field>
void init(Field& u)
{
    auto& mesh = u.mesh();
    u.resize();
    samurai::for_each_cell(mesh,
                           [&](auto& cell)
                           {
                               auto center    = cell.center();
                               const double x = center[0], y = center[1];
                               const bool in_disc   = (x - 0.3) * (x - 0.3) + (y - 0.3) * (y - 0.3) <= 0.2 * 0.2;
                               const bool in_square = x >= 0.5 && x <= 0.7 && y >= 0.4 && y <= 0.6;
                               u[cell]              = std::array<double, 2>{in_disc ? 1. : 0., 0.};
                               u[cell][1]           = in_square ? 0.5 : 0.;
                           });
}

int main(int argc, char** argv)
{
    if (argc < 2)
    {
        std::fprintf(stderr, "usage: vector_advection_2d <out.txt> [relative]\n");
        return 2;
    }
    const bool relative = argc > 2 && std::string(argv[2]) == "relative";
    try
    {
        constexpr std::size_t dim = 2;
        std::array<double, dim> a{{1, 0.5}};
        const samurai::Box<double, dim> box({0., 0.}, {1., 1.});
        auto config = samurai::mesh_config<dim>().min_level(3).max_level(8).max_stencil_size(2).disable_minimal_ghost_width();
        auto mesh   = samurai::mra::make_mesh(box, config);
        auto u      = samurai::make_vector_field<double, 2>("u", mesh);
        init(u);
        samurai::make_bc<samurai::Dirichlet<1>>(u, 0., 0.25);
        auto unp1 = samurai::make_vector_field<double, 2>("unp1", mesh);

        const double dt   = 0.5 * mesh.min_cell_length();
        auto MRadaptation = samurai::make_MRAdapt(u);
        auto mra_config   = samurai::mra_config().epsilon(1e-3).relative_detail(relative);
        const std::size_t n_steps = 12;
        for (std::size_t nt = 0; nt < n_steps; ++nt)
        {
            MRadaptation(mra_config);
            samurai::update_ghost_mr(u);
            unp1.resize();
            unp1 = u - dt * samurai::upwind(a, u);
            std::swap(u.array(), unp1.array());
        }

        FILE* f = std::fopen(argv[1], "w");
        if (!f)
        {
            return 1;
        }
        std::fprintf(f, "%zu\n", n_steps);
        samurai::for_each_cell(mesh,
                               [&](auto& cell)
                               {
                                   const auto v = static_cast<const decltype(u)&>(u)[cell];
                                   std::fprintf(f, "%zu %d %d %.17g %.17g\n", cell.level, cell.indices[0], cell.indices[1], v[0], v[1]);
                               });
        std::fclose(f);
        return 0;
    }
    catch (const std::exception& e)
    {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
}
