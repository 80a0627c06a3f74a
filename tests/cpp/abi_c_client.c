/* A plain C client of the C ABI: compiles as C99 against include/samurai_gpu.h and links against
 * libsamurai_gpu.so (the CPU test builds it; it needs a GPU to run).  It makes the loop body of samurai's
 * advection demo (adapt, ghost update, upwind, swap) through the C calls, then reads the leaf values back. */
#include <stdio.h>
#include <stdlib.h>

#include "samurai_gpu.h"

static int check(int st, const char* what)
{
    if (st != SG_OK)
    {
        fprintf(stderr, "%s: status %d: %s\n", what, st, sg_last_error());
    }
    return st;
}

int main(void)
{
    sg_mesh_t mesh   = NULL;
    sg_field_t u     = NULL;
    sg_field_t unp1  = NULL;
    const double a[3] = {1.0, 1.0, 0.0};
    const double dt   = 0.5 / 256.0;
    long long nc = 0, nref = 0;
    int passes = 0;
    if (check(sg_mesh_create(2, 2, 8, 1, 1, 1, &mesh), "sg_mesh_create") || check(sg_field_create(mesh, "u", &u), "sg_field_create")
        || check(sg_field_create(mesh, "unp1", &unp1), "sg_field_create") || check(sg_field_set_dirichlet(u, 0.0), "sg_field_set_dirichlet"))
    {
        return 1;
    }
    for (int it = 0; it < 4; ++it)
    {
        if (check(sg_step(u, unp1, 1e-4, 2.0, a, dt, SG_UPWIND_OP, &passes), "sg_step"))
        {
            return 1;
        }
    }
    if (check(sg_mesh_counts(mesh, &nc, &nref), "sg_mesh_counts"))
    {
        return 1;
    }
    double* values = (double*)malloc(sizeof(double) * (size_t)(nc > 0 ? nc : 1));
    if (!values || check(sg_field_get_cells(u, values, nc), "sg_field_get_cells"))
    {
        return 1;
    }
    printf("%lld leaf cells after %d steps\n", nc, 4);
    free(values);
    sg_field_destroy(unp1);
    sg_field_destroy(u);
    sg_mesh_destroy(mesh);
    return 0;
}
