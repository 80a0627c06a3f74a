// demos/FiniteVolume/advection_2d.cpp of samurai, written against the
// GB300 drop-in header: the samurai calls are the demo's own (the output and
// CLI parts are replaced by printing the final cells).  Usage:
//   advection_2d <pred 0|1> <out.txt> [upwind|convection|periodic [<dir> <name>]]
// With "convection" the step is the flux form of
// demos/FiniteVolume/linear_convection.cpp: unp1 = u - dt * conv(u) with
// conv = make_convection_upwind<decltype(u)>(a); "periodic" runs the upwind
// operator on a mesh periodic along both axes (mesh_config::periodic(true)).
// With <dir> <name> the final
// state is also written as the demo's save() does (samurai::save(path,
// filename, mesh, u), advection_2d.cpp:46-66) and as a restart file
// (samurai::dump), then read back with samurai::load.
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
                               auto center           = cell.center();
                               const double radius   = .2;
                               const double x_center = 0.3;
                               const double y_center = 0.3;
                               if (((center[0] - x_center) * (center[0] - x_center) + (center[1] - y_center) * (center[1] - y_center))
                                   <= radius * radius)
                               {
                                   u[cell] = 1;
                               }
                               else
                               {
                                   u[cell] = 0;
                               }
                           });
}

// mode "default": samurai's default mesh configuration (no disable_minimal_ghost_width(): max_stencil_radius 2),
// "refine_boundary": the same with samurai::args::refine_boundary (--refine-boundary)
template <int pred>
int run(const char* out_path, bool flux_form, bool periodic, bool default_config, const char* save_dir, const char* save_name)
{
    constexpr std::size_t dim = 2;
    std::array<double, dim> a{{1, 1}};
    double Tf  = .01;
    double cfl = 0.5;
    double t   = 0.;

    const samurai::Box<double, dim> box({0., 0.}, {1., 1.});
    auto config = samurai::mesh_config<dim, pred>().min_level(4).max_level(10);
    if (!default_config)
    {
        config.max_stencil_size(2).disable_minimal_ghost_width();
    }
    if (periodic)
    {
        config.periodic(true);
    }
    auto mesh   = samurai::mra::make_mesh(box, config);
    auto u      = samurai::make_scalar_field<double>("u", mesh);
    init(u);
    samurai::make_bc<samurai::Dirichlet<1>>(u, 0.);

    double dt = cfl * mesh.min_cell_length();
    auto unp1 = samurai::make_scalar_field<double>("unp1", mesh);

    auto MRadaptation = samurai::make_MRAdapt(u);
    auto mra_config   = samurai::mra_config().epsilon(2e-4);
    MRadaptation(mra_config);

    std::size_t nt = 0;
    while (t != Tf)
    {
        MRadaptation(mra_config);
        t += dt;
        if (t > Tf)
        {
            dt += Tf - t;
            t = Tf;
        }
        samurai::update_ghost_mr(u);
        unp1.resize();
        if (flux_form)
        {
            samurai::VelocityVector<dim> velocity = {a[0], a[1]};
            auto conv                             = samurai::make_convection_upwind<decltype(u)>(velocity);
            unp1                                  = u - dt * conv(u);
        }
        else
        {
            unp1 = u - dt * samurai::upwind(a, u);
        }
        std::swap(u.array(), unp1.array());
        ++nt;
    }

    if (save_dir)
    {
        samurai::save(save_dir, save_name, mesh, u);
        samurai::dump(save_dir, std::string(save_name) + "_restart", mesh, u);
        auto mesh2 = samurai::mra::make_mesh(box, config);
        auto u2    = samurai::make_scalar_field<double>("u", mesh2);
        samurai::load(save_dir, std::string(save_name) + "_restart", mesh2, u2);
        std::size_t n1 = 0, n2 = 0, same = 0;
        samurai::for_each_cell(mesh, [&](auto&) { ++n1; });
        auto c1         = mesh.cells();
        auto c2         = mesh2.cells();
        const auto& cu  = u;
        const auto& cu2 = u2;
        n2              = c2.size();
        for (std::size_t k = 0; k < n1 && k < n2; ++k)
        {
            same += (c1[k].level == c2[k].level && c1[k].indices == c2[k].indices && cu[c1[k]] == cu2[c2[k]]) ? 1 : 0;
        }
        if (n1 != n2 || same != n1)
        {
            std::fprintf(stderr, "restart differs: %zu cells, %zu loaded, %zu equal\n", n1, n2, same);
            return 1;
        }
    }

    FILE* f = std::fopen(out_path, "w");
    if (!f)
    {
        return 1;
    }
    std::fprintf(f, "%zu\n", nt);
    samurai::for_each_cell(mesh,
                           [&](auto& cell) { std::fprintf(f, "%zu %d %d %.17g\n", cell.level, cell.indices[0], cell.indices[1], u[cell]); });
    std::fclose(f);
    return 0;
}

int main(int argc, char** argv)
{
    if (argc < 3)
    {
        std::fprintf(stderr, "usage: advection_2d <pred 0|1> <out.txt> [upwind|convection|periodic|default|refine_boundary [<dir> <name>]]\n");
        return 2;
    }
    const std::string mode = argc > 3 ? argv[3] : "";
    const bool flux_form   = mode == "convection";
    const bool periodic    = mode == "periodic";
    const bool dflt        = mode == "default" || mode == "refine_boundary";
    samurai::args::refine_boundary = mode == "refine_boundary";
    const char* save_dir  = argc > 5 ? argv[4] : nullptr;
    const char* save_name = argc > 5 ? argv[5] : nullptr;
    try
    {
        return std::atoi(argv[1]) == 0 ? run<0>(argv[2], flux_form, periodic, dflt, save_dir, save_name)
                                       : run<1>(argv[2], flux_form, periodic, dflt, save_dir, save_name);
    }
    catch (const std::exception& e)
    {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
}
