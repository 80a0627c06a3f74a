// FP64 kernels of the MR advection step on the dense level slabs:
// update_ghost_mr (outer ghosts, projection, prediction), wavelet details,
// keep/coarsen/refine criteria, tag finalisation, update_fields and the
// first-order upwind step.  Built with --fmad=false: every FP64 operation is
// rounded on its own, in the reference's association order, so that the
// detail thresholds take the same decisions as the CPU implementation.
#include "sg_ctx.cuh"

namespace sg
{
    // set by kernels that met a position outside the stored box
    __device__ int sg_device_error = 0;

    int device_error(Ctx& c)
    {
        int v = 0;
        if (cudaMemcpyFromSymbolAsync(&v, sg_device_error, sizeof(int), 0, cudaMemcpyDeviceToHost, c.stream) != cudaSuccess
            || cudaStreamSynchronize(c.stream) != cudaSuccess)
        {
            return check(c, "device_error");
        }
        if (v)
        {
            const int zero = 0;
            cudaMemcpyToSymbolAsync(sg_device_error, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, c.stream);
            c.err = "a kernel addressed a cell outside the stored level box (invalid mesh)";
            return SG_ERR_STATE;
        }
        return SG_OK;
    }

    int new_cells_from_tags(Ctx& c, const DeviceMesh& m, uint32_t* nc);
    int graduate(Ctx& c, uint32_t* nc, int* iterations);
    int bitmaps_equal(Ctx& c, const uint32_t* a, const uint32_t* b, bool* equal);

    namespace
    {
        constexpr int BLOCK = 256;

        // Warp-cooperative traversal of the set bits of a computed subset:
        // lane k evaluates word c0+k, the warp then visits every non-empty
        // word with one lane per bit, so field accesses are 256 B coalesced.
        template <class WordF, class CellF>
        __device__ __forceinline__ void warp_bits(long long wb, long long we, WordF word_of, CellF cell)
        {
            const int lane         = threadIdx.x & 31;
            const long long warp   = (blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x) >> 5;
            const long long nwarps = (static_cast<long long>(gridDim.x) * blockDim.x) >> 5;
            for (long long c0 = wb + warp * 32; c0 < we; c0 += nwarps * 32)
            {
                const long long w = c0 + lane;
                const uint32_t v  = (w < we) ? word_of(w) : 0u;
                uint32_t nz       = __ballot_sync(0xffffffffu, v != 0u);
                while (nz)
                {
                    const int j = __ffs(nz) - 1;
                    nz &= nz - 1;
                    const uint32_t vj = __shfl_sync(0xffffffffu, v, j);
                    if ((vj >> lane) & 1u)
                    {
                        cell(c0 + j, lane);
                    }
                }
            }
        }

        // interp_coeffs<3> (numeric/prediction.hpp:32-36), parity 0: even
        __device__ __forceinline__ double interp1(int parity, int k)
        {
            const double sign = parity ? -1. : 1.;
            return k == 0 ? sign / 8. : (k == 1 ? 1. : -sign / 8.);
        }

        // Element of a cell that the reference algorithm guarantees to be in
        // the stored box.  A position outside it (a bug or an invalid mesh)
        // is recorded in the device error word and redirected to element 0,
        // so that no access leaves the allocation.
        __device__ __forceinline__ long long elem_at(const Geom& g, int l, int x, int y, int z)
        {
            const Pos p = pos_of(g, l, x, y, z);
            if (p.w < 0)
            {
                atomicOr(&sg_device_error, 1);
                return 0;
            }
            return elem(p);
        }

        // prediction_op<order,false> for one fine cell (numeric/prediction.hpp:286-361)
        __device__ __forceinline__ double predict_one(const Geom& g, const double* u, int l, int x, int y, int z, int order)
        {
            const int px = x >> 1, py = y >> 1, pz = z >> 1;
            if (order == 0)
            {
                return u[elem_at(g, l - 1, px, py, pz)];
            }
            double acc  = 0.;
            const int nz = (g.dim == 3) ? 3 : 1;
            for (int sz = 0; sz < nz; ++sz)
            {
                for (int sy = 0; sy < 3; ++sy)
                {
                    const long long base = elem_at(g, l - 1, px - 1, py + sy - 1, (g.dim == 3) ? pz + sz - 1 : 0);
                    for (int sx = 0; sx < 3; ++sx)
                    {
                        double coeff = 1.;
                        coeff        = coeff * interp1(x & 1, sx);
                        coeff        = coeff * interp1(y & 1, sy);
                        if (g.dim == 3)
                        {
                            coeff = coeff * interp1(z & 1, sz);
                        }
                        acc = acc + u[base + sx] * coeff;
                    }
                }
            }
            return acc;
        }

        // projection_op_ (numeric/projection.hpp:15-65)
        __device__ __forceinline__ double project_one(const Geom& g, const double* u, int lf, int x, int y, int z)
        {
            double sum   = 0.;
            const int nz = (g.dim == 3) ? 2 : 1;
            for (int sz = 0; sz < nz; ++sz)
            {
                for (int sy = 0; sy < 2; ++sy)
                {
                    const long long e = elem_at(g, lf, 2 * x, 2 * y + sy, (g.dim == 3) ? 2 * z + sz : 0);
                    sum               = sum + (u[e] + u[e + 1]);
                }
            }
            const double inv = (g.dim == 3) ? 0.125 : 0.25;
            return sum * inv;
        }

        // ----------------------------------------------------------- tags
        __global__ void k_tag_init(Geom g, const uint32_t* ref, const uint32_t* cells, uint8_t* tag, double* det)
        {
            warp_bits(0, g.total_words, [=](long long w) { return ref[w]; },
                      [=](long long w, int b)
                      {
                          const long long e = 32 * w + b;
                          tag[e]            = static_cast<uint8_t>((cells[w] >> b) & 1u);
                          det[e]            = 0.;
                      });
        }

        // ----------------------------------------------------- outer ghosts
        struct Dirs
        {
            int n;
            int d[26][3];
        };

        // for_each_diagonal_direction order (stencil.hpp:338-349)
        Dirs diagonal_dirs(int dim)
        {
            Dirs out{};
            for (int z = (dim == 3 ? -1 : 0); z <= (dim == 3 ? 1 : 0); ++z)
            {
                for (int y = -1; y <= 1; ++y)
                {
                    for (int x = -1; x <= 1; ++x)
                    {
                        const int nnz = (x != 0) + (y != 0) + (z != 0);
                        if (nnz > 1)
                        {
                            out.d[out.n][0] = x;
                            out.d[out.n][1] = y;
                            out.d[out.n][2] = z;
                            ++out.n;
                        }
                    }
                }
            }
            return out;
        }

        // update_outer_corners_by_polynomial_extrapolation for a ghost width
        // of 1 (bc/apply_field_bc.hpp:371-505) followed by project_corner_below
        // (algorithm/update_outer_ghost.hpp:268-337).  One block per direction.
        __global__ void k_corners(Geom g, Dirs dirs, int l, const uint32_t* cells, const uint32_t* ref, double* u)
        {
            const int* d  = dirs.d[blockIdx.x];
            const int n   = g.lv[l].n;
            int nfree     = 0;
            for (int k = 0; k < g.dim; ++k)
            {
                nfree += (d[k] == 0);
            }
            const long long npos = (nfree == 0) ? 1 : n; // 3D edges have one free axis
            for (long long t = threadIdx.x; t < npos; t += blockDim.x)
            {
                int c[3];
                for (int k = 0; k < 3; ++k)
                {
                    c[k] = (k < g.dim) ? (d[k] > 0 ? n - 1 : (d[k] < 0 ? 0 : static_cast<int>(t))) : 0;
                }
                const Pos pc = pos_of(g, l, c[0], c[1], c[2]);
                if (test(cells, pc))
                {
                    const long long eg = elem_at(g, l, c[0] + d[0], c[1] + d[1], g.dim == 3 ? c[2] + d[2] : 0);
                    u[eg]              = u[elem(pc)];
                }
            }
            __syncthreads();
            for (int dl = 1; dl <= 2; ++dl)
            {
                const int pl = l - dl;
                if (pl < 0)
                {
                    break;
                }
                const int npl          = g.lv[pl].n;
                const long long npos_c = (nfree == 0) ? 1 : npl;
                for (long long t = threadIdx.x; t < npos_c; t += blockDim.x)
                {
                    int gc[3], ch[3];
                    for (int k = 0; k < 3; ++k)
                    {
                        if (k >= g.dim)
                        {
                            gc[k] = ch[k] = 0;
                            continue;
                        }
                        gc[k] = d[k] > 0 ? npl : (d[k] < 0 ? -1 : static_cast<int>(t));
                        ch[k] = (gc[k] << dl) + (d[k] == -1 ? ((1 << dl) - 1) : 0);
                    }
                    const Pos pg = pos_of(g, pl, gc[0], gc[1], gc[2]);
                    const Pos pf = pos_of(g, l, ch[0], ch[1], ch[2]);
                    if (test(ref, pg) && test(ref, pf))
                    {
                        u[elem(pg)] = u[elem(pf)];
                    }
                }
            }
        }

        // face position helper: direction index k in 0..2*dim-1 is
        // (+e0,-e0,+e1,-e1,...) (stencil.hpp:301-317)
        __device__ __forceinline__ void face_cell(const Geom& g, int l, int k, long long t, int* in, int* dir)
        {
            const int axis = k >> 1;
            const int sgn  = (k & 1) ? -1 : 1;
            const int n    = g.lv[l].n;
            int free_[2]   = {static_cast<int>(t % n), static_cast<int>(t / n)};
            int f          = 0;
            for (int a = 0; a < 3; ++a)
            {
                dir[a] = 0;
                if (a >= g.dim)
                {
                    in[a] = 0;
                    continue;
                }
                if (a == axis)
                {
                    in[a] = sgn > 0 ? n - 1 : 0;
                    dir[a] = sgn;
                }
                else
                {
                    in[a] = free_[f++];
                }
            }
        }

        // project_bc (algorithm/update_outer_ghost.hpp:20-155) and the
        // Dirichlet<1> ghost u_g = 2 v - u_c (bc/dirichlet.hpp:22-29) for every
        // Cartesian direction at level l.
        __global__ void k_faces(Geom g, int l, int do_project, int do_dirichlet, double value, const uint32_t* cells, const uint32_t* uni,
                                const uint32_t* ref, double* u)
        {
            const int n          = g.lv[l].n;
            const long long nf   = (g.dim == 2) ? n : static_cast<long long>(n) * n;
            const long long ntot = nf * 2 * g.dim;
            for (long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; t < ntot; t += static_cast<long long>(gridDim.x) * blockDim.x)
            {
                const int k = static_cast<int>(t / nf);
                int in[3], dir[3];
                face_cell(g, l, k, t - k * nf, in, dir);
                const Pos pi = pos_of(g, l, in[0], in[1], in[2]);
                const int gx = in[0] + dir[0], gy = in[1] + dir[1], gz = in[2] + dir[2];
                if (do_dirichlet && test(cells, pi))
                {
                    const long long eg = elem_at(g, l, gx, gy, gz);
                    u[eg]              = 2 * value - u[elem(pi)];
                }
                else if (do_project && test(uni, pi))
                {
                    const Pos pg = pos_of(g, l, gx, gy, gz);
                    if (!test(ref, pg))
                    {
                        continue;
                    }
                    double sum = 0.;
                    int nch    = 0;
                    for (int dl = 1; dl <= 2 && nch == 0; ++dl)
                    {
                        const int lc = l + dl;
                        const int m  = 1 << dl;
                        for (int sz = 0; sz < (g.dim == 3 ? m : 1); ++sz)
                        {
                            for (int sy = 0; sy < m; ++sy)
                            {
                                for (int sx = 0; sx < m; ++sx)
                                {
                                    const Pos pc = pos_of(g, lc, gx * m + sx, gy * m + sy, g.dim == 3 ? gz * m + sz : 0);
                                    if (test(ref, pc))
                                    {
                                        sum = sum + u[elem(pc)];
                                        ++nch;
                                    }
                                }
                            }
                        }
                    }
                    u[elem(pg)] = nch > 0 ? sum / static_cast<double>(nch) : 0.;
                }
            }
        }

        // predict_bc (algorithm/update_outer_ghost.hpp:195-266): the children
        // at l+1 of the Dirichlet ghosts of level l copy their parent.
        __global__ void k_faces_predict(Geom g, int l, const uint32_t* cells, const uint32_t* ref, double* u)
        {
            const int n          = g.lv[l].n;
            const long long nf   = (g.dim == 2) ? n : static_cast<long long>(n) * n;
            const long long ntot = nf * 2 * g.dim;
            for (long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; t < ntot; t += static_cast<long long>(gridDim.x) * blockDim.x)
            {
                const int k = static_cast<int>(t / nf);
                int in[3], dir[3];
                face_cell(g, l, k, t - k * nf, in, dir);
                if (!test(cells, g, l, in[0], in[1], in[2]))
                {
                    continue;
                }
                const int px = in[0] + dir[0], py = in[1] + dir[1], pz = in[2] + dir[2];
                const double v = u[elem_at(g, l, px, py, pz)];
                for (int sz = 0; sz < (g.dim == 3 ? 2 : 1); ++sz)
                {
                    for (int sy = 0; sy < 2; ++sy)
                    {
                        for (int sx = 0; sx < 2; ++sx)
                        {
                            const Pos pf = pos_of(g, l + 1, 2 * px + sx, 2 * py + sy, g.dim == 3 ? 2 * pz + sz : 0);
                            if (test(ref, pf))
                            {
                                u[elem(pf)] = v;
                            }
                        }
                    }
                }
            }
        }

        // projection of the reference cells of level l onto proj_cells[l-1]
        // (algorithm/update_ghost_mr.hpp:217-221)
        __global__ void k_project(Geom g, int l, const uint32_t* proj, const uint32_t* ref, double* u)
        {
            const int lc = l - 1;
            warp_bits(g.lv[lc].woff, g.lv[lc].woff + g.lv[lc].nwords,
                      [=](long long w)
                      {
                          const WordLoc loc = word_loc(g, lc, w);
                          return proj[w] & coarsen_word(g, ref, lc, loc.row, loc.wi);
                      },
                      [=](long long w, int b)
                      {
                          const Cell c = cell_of(g, lc, w, b);
                          u[32 * w + b] = project_one(g, u, l, c.x, c.y, c.z);
                      });
        }

        // prediction of the ghosts of level l from level l-1
        // (algorithm/update_ghost_mr.hpp:224-233)
        __global__ void k_predict(Geom g, int l, int order, const uint32_t* cells, const uint32_t* proj, const uint32_t* ref, double* u)
        {
            warp_bits(g.lv[l].woff, g.lv[l].woff + g.lv[l].nwords,
                      [=](long long w)
                      {
                          const WordLoc loc = word_loc(g, l, w);
                          return ref[w] & ~(cells[w] | proj[w]) & box_mask(g, l, loc.row, loc.wi, 0, 0) & refine_word(g, ref, l, loc.row, loc.wi);
                      },
                      [=](long long w, int b)
                      {
                          const Cell c = cell_of(g, l, w, b);
                          u[32 * w + b] = predict_one(g, u, l, c.x, c.y, c.z, order);
                      });
        }

        // -------------------------------------------------------- details
        // compute_detail_op (mr/operators.hpp:139-540) on
        // intersection(all_cells[l], union(cells[l+1], cells[l+2])).on(l)
        __global__ void k_detail(Geom g, int l0, int l1, int order, const uint32_t* ref, const uint32_t* hc, const uint32_t* hc2, const double* u,
                                 double* det)
        {
            warp_bits(g.lv[l0].woff, g.lv[l1].woff + g.lv[l1].nwords, [=](long long w) { return ref[w] & (hc[w] | hc2[w]); },
                      [=](long long w, int b)
                      {
                          const int l    = level_of(g, w);
                          const Cell c   = cell_of(g, l, w, b);
                          const int nch  = 1 << g.dim;
                          long long ce[8];
                          for (int ch = 0; ch < nch; ++ch)
                          {
                              ce[ch] = elem_at(g, l + 1, 2 * c.x + (ch & 1), 2 * c.y + ((ch >> 1) & 1), g.dim == 3 ? 2 * c.z + ((ch >> 2) & 1) : 0);
                          }
                          if (order == 0)
                          {
                              const double uc = u[32 * w + b];
                              for (int ch = 0; ch < nch; ++ch)
                              {
                                  det[ce[ch]] = u[ce[ch]] - uc;
                              }
                              return;
                          }
                          double d[8];
                          for (int ch = 0; ch < nch; ++ch)
                          {
                              d[ch] = u[ce[ch]];
                          }
                          const int nz = (g.dim == 3) ? 3 : 1;
                          for (int sz = 0; sz < nz; ++sz)
                          {
                              for (int sy = 0; sy < 3; ++sy)
                              {
                                  const long long base = elem_at(g, l, c.x - 1, c.y + sy - 1, g.dim == 3 ? c.z + sz - 1 : 0);
                                  for (int sx = 0; sx < 3; ++sx)
                                  {
                                      const double src = u[base + sx];
                                      for (int ch = 0; ch < nch; ++ch)
                                      {
                                          double cf = interp1(ch & 1, sx) * interp1((ch >> 1) & 1, sy);
                                          if (g.dim == 3)
                                          {
                                              cf = cf * interp1((ch >> 2) & 1, sz);
                                          }
                                          d[ch] = d[ch] - cf * src;
                                      }
                                  }
                              }
                          }
                          for (int ch = 0; ch < nch; ++ch)
                          {
                              det[ce[ch]] = d[ch];
                          }
                      });
        }

        struct Eps
        {
            double eps[MAXLEV];    // eps_l, indexed by the fine level
            double fine[MAXLEV];   // 2^(reg+dim) * eps_l
            double coarse[MAXLEV]; // fine / 2^dim
        };

        // mr_criteria_op (mr/criteria.hpp:20-113) on
        // intersection(cells[l], all_cells[l-1]).on(l-1), fine levels l0..l1
        __global__ void k_criteria(Geom g, int l0, int l1, Eps eps, const uint32_t* ref, const uint32_t* hc, const double* det, uint8_t* tag)
        {
            const int lc0 = l0 - 1, lc1 = l1 - 1;
            warp_bits(g.lv[lc0].woff, g.lv[lc1].woff + g.lv[lc1].nwords, [=](long long w) { return ref[w] & hc[w]; },
                      [=](long long w, int b)
                      {
                          const int lc  = level_of(g, w);
                          const int lf  = lc + 1;
                          const Cell c  = cell_of(g, lc, w, b);
                          const int nch = 1 << g.dim;
                          long long fo[8];
                          for (int ch = 0; ch < nch; ++ch)
                          {
                              fo[ch] = elem_at(g, lf, 2 * c.x + (ch & 1), 2 * c.y + ((ch >> 1) & 1), g.dim == 3 ? 2 * c.z + ((ch >> 2) & 1) : 0);
                          }
                          if (lf > g.min_level)
                          {
                              const bool cond = fabs(det[32 * w + b]) > eps.coarse[lf];
                              if (!cond)
                              {
                                  bool ok = true;
                                  for (int ch = 0; ch < nch; ++ch)
                                  {
                                      if (fabs(det[fo[ch]]) > eps.eps[lf])
                                      {
                                          ok = false;
                                          break;
                                      }
                                  }
                                  if (ok)
                                  {
                                      for (int ch = 0; ch < nch; ++ch)
                                      {
                                          tag[fo[ch]] = 2;
                                      }
                                  }
                              }
                          }
                          if (lf < g.max_level)
                          {
                              for (int ch = 0; ch < nch; ++ch)
                              {
                                  if (fabs(det[fo[ch]]) > eps.fine[lf])
                                  {
                                      tag[fo[ch]] |= 4;
                                  }
                              }
                          }
                      });
        }

        // maximum_op (mr/operators.hpp:22-96), children at level l
        __global__ void k_maximum(Geom g, int l, const uint32_t* ref, const uint32_t* hc, uint8_t* tag)
        {
            const int lc = l - 1;
            warp_bits(g.lv[lc].woff, g.lv[lc].woff + g.lv[lc].nwords, [=](long long w) { return ref[w] & hc[w]; },
                      [=](long long w, int b)
                      {
                          const Cell c  = cell_of(g, lc, w, b);
                          const int nch = 1 << g.dim;
                          long long fo[8];
                          uint8_t keep = 0, coarsen = 2;
                          for (int ch = 0; ch < nch; ++ch)
                          {
                              fo[ch] = elem_at(g, l, 2 * c.x + (ch & 1), 2 * c.y + ((ch >> 1) & 1), g.dim == 3 ? 2 * c.z + ((ch >> 2) & 1) : 0);
                              const uint8_t t = tag[fo[ch]];
                              keep |= t & 1;
                              coarsen &= t & 2;
                          }
                          const long long co = 32 * w + b;
                          if (keep)
                          {
                              for (int ch = 0; ch < nch; ++ch)
                              {
                                  tag[fo[ch]] |= 1;
                              }
                              tag[co] |= 1;
                          }
                          else if (coarsen)
                          {
                              tag[co] |= 1;
                          }
                          else
                          {
                              for (int ch = 0; ch < nch; ++ch)
                              {
                                  tag[fo[ch]] &= static_cast<uint8_t>(~2);
                              }
                          }
                      });
        }

        // update_fields (algorithm/update_fields.hpp:27-127): copy on
        // reference ∩ new cells, projection on coarsened cells, prediction on
        // refined cells; every other reference entry of the new field is 0.
        __global__ void k_update_fields(Geom g, int order, const uint32_t* nref, const uint32_t* ncells, const uint32_t* oref, const uint32_t* ocells,
                                        const uint32_t* ohc, const double* uo, double* un)
        {
            warp_bits(0, g.total_words, [=](long long w) { return nref[w]; },
                      [=](long long w, int b)
                      {
                          const long long e = 32 * w + b;
                          double v          = 0.;
                          if ((ncells[w] >> b) & 1u)
                          {
                              const int l  = level_of(g, w);
                              const Cell c = cell_of(g, l, w, b);
                              if ((ohc[w] >> b) & 1u)
                              {
                                  v = project_one(g, uo, l + 1, c.x, c.y, c.z);
                              }
                              else if (l >= 1 && test(ocells, g, l - 1, c.x >> 1, c.y >> 1, c.z >> 1))
                              {
                                  v = predict_one(g, uo, l, c.x, c.y, c.z, order);
                              }
                              else if ((oref[w] >> b) & 1u)
                              {
                                  v = uo[e];
                              }
                          }
                          un[e] = v;
                      });
        }

        // -------------------------------------------------------- upwind
        // unp1 = u - dt * upwind(a, u) (stencil_field.hpp:38-44, 91-97;
        // demos/FiniteVolume/advection_2d.cpp:144) or the README lambda
        // (README.md:144-153).  Neighbours at the same level are reference
        // cells, at fixed offsets in the dense slabs.
        __global__ void k_upwind(Geom g, const uint32_t* cells, const double* u, double* unp1, double a0, double a1, double a2, double dt, int scheme)
        {
            warp_bits(0, g.total_words, [=](long long w) { return cells[w]; },
                      [=](long long w, int b)
                      {
                          const int l          = level_of(g, w);
                          const LevelGeom& L   = g.lv[l];
                          const long long e    = 32 * w + b;
                          const long long sy   = 32LL * L.W;
                          const long long sz   = sy * L.R;
                          const double dx      = 1.0 / static_cast<double>(1 << l);
                          const double uc      = u[e];
                          double out;
                          if (scheme == 1)
                          {
                              double s = uc - u[e - 1];
                              s        = s + uc;
                              s        = s - u[e - sy];
                              if (g.dim == 3)
                              {
                                  s = s + uc;
                                  s = s - u[e - sz];
                              }
                              out = uc - dt / dx * s;
                          }
                          else
                          {
                              const double ha0 = .5 * a0, hb0 = .5 * fabs(a0);
                              const double ha1 = .5 * a1, hb1 = .5 * fabs(a1);
                              const double ul = u[e - 1], ur = u[e + 1], ud = u[e - sy], uu = u[e + sy];
                              const double lf = ha0 * (ul + uc) + hb0 * (ul - uc);
                              const double rf = ha0 * (uc + ur) + hb0 * (uc - ur);
                              const double df = ha1 * (ud + uc) + hb1 * (ud - uc);
                              const double uf = ha1 * (uc + uu) + hb1 * (uc - uu);
                              double s        = -lf + rf;
                              s               = s + -df;
                              s               = s + uf;
                              if (g.dim == 3)
                              {
                                  const double ha2 = .5 * a2, hb2 = .5 * fabs(a2);
                                  const double uf2 = u[e - sz], ub2 = u[e + sz];
                                  const double ff  = ha2 * (uf2 + uc) + hb2 * (uf2 - uc);
                                  const double bf  = ha2 * (uc + ub2) + hb2 * (uc - ub2);
                                  s                = s + -ff;
                                  s                = s + bf;
                              }
                              const double up = s / dx;
                              out             = uc - dt * up;
                          }
                          unp1[e] = out;
                      });
        }

        // --------------------------------------------------- layout moves
        __global__ void k_gather(Geom g, const uint32_t* ref, const int* rank, const double* dense, double* compact)
        {
            warp_bits(0, g.total_words, [=](long long w) { return ref[w]; },
                      [=](long long w, int b) { compact[ref_index(ref, rank, Pos{w, b})] = dense[32 * w + b]; });
        }

        __global__ void k_scatter(Geom g, const uint32_t* ref, const int* rank, const double* compact, double* dense)
        {
            warp_bits(0, g.total_words, [=](long long w) { return ref[w]; },
                      [=](long long w, int b) { dense[32 * w + b] = compact[ref_index(ref, rank, Pos{w, b})]; });
        }

        __global__ void k_fill(Geom g, const uint32_t* ref, double* dense, double v)
        {
            warp_bits(0, g.total_words, [=](long long w) { return ref[w]; }, [=](long long w, int b) { dense[32 * w + b] = v; });
        }

        int grid_words(long long nwords)
        {
            // one warp per 32 words, capped at 8 resident blocks per SM
            return grid_for((nwords + 31) / 32 * 32, BLOCK, 152LL * 8);
        }
    } // namespace

    int gather_compact(Ctx& c, const DeviceMesh& m, const double* dense, double* compact)
    {
        k_gather<<<grid_words(c.g.total_words), BLOCK, 0, c.stream>>>(c.g, m.ref, m.rank, dense, compact);
        ++c.n_launches;
        return check(c, "gather");
    }

    int scatter_compact(Ctx& c, const DeviceMesh& m, const double* compact, double* dense)
    {
        k_scatter<<<grid_words(c.g.total_words), BLOCK, 0, c.stream>>>(c.g, m.ref, m.rank, compact, dense);
        ++c.n_launches;
        return check(c, "scatter");
    }

    int fill_ref(Ctx& c, const DeviceMesh& m, double* dense, double value)
    {
        k_fill<<<grid_words(c.g.total_words), BLOCK, 0, c.stream>>>(c.g, m.ref, dense, value);
        ++c.n_launches;
        return check(c, "fill");
    }

    // update_ghost_mr / update_ghost_mr_aggregated (algorithm/update_ghost_mr.hpp:195-270)
    int update_ghost_mr(Ctx& c, DeviceField& f)
    {
        const Geom& g   = c.g;
        DeviceMesh& m   = c.m();
        const int minl  = c.cfg.min_level;
        const int maxl  = c.cfg.max_level;
        const int lmin  = minl >= 2 ? minl - 2 : 0; // no reference cell below min_level-2
        double* u       = f.data;
        static const Dirs diag2 = diagonal_dirs(2);
        static const Dirs diag3 = diagonal_dirs(3);
        const Dirs& diag        = (g.dim == 2) ? diag2 : diag3;
        if (c.cfg.ghost_width != 1)
        {
            c.err = "update_ghost_mr: only a ghost width of 1 is implemented";
            return SG_ERR_ARG;
        }
        for (int l = maxl; l >= lmin; --l)
        {
            if (l >= minl && l <= maxl)
            {
                k_corners<<<diag.n, BLOCK, 0, c.stream>>>(g, diag, l, m.cells, m.ref, u);
                ++c.n_launches;
            }
            const int n       = g.lv[l].n;
            const long long nf = static_cast<long long>(2 * g.dim) * ((g.dim == 2) ? n : static_cast<long long>(n) * n);
            const int do_proj = l < maxl;
            const int do_bc   = (l >= minl) && f.has_bc;
            if (do_proj || do_bc)
            {
                k_faces<<<grid_for(nf), BLOCK, 0, c.stream>>>(g, l, do_proj, do_bc, f.bc_value, m.cells, m.uni, m.ref, u);
                ++c.n_launches;
            }
            if (l >= minl && l < maxl)
            {
                k_faces_predict<<<grid_for(nf), BLOCK, 0, c.stream>>>(g, l, m.cells, m.ref, u);
                ++c.n_launches;
            }
            if (l > lmin)
            {
                k_project<<<grid_words(g.lv[l - 1].nwords), BLOCK, 0, c.stream>>>(g, l, m.proj, m.ref, u);
                ++c.n_launches;
            }
        }
        for (int l = 1; l <= maxl; ++l)
        {
            if (l < lmin)
            {
                continue;
            }
            k_predict<<<grid_words(g.lv[l].nwords), BLOCK, 0, c.stream>>>(g, l, c.cfg.prediction_radius, m.cells, m.proj, m.ref, u);
            ++c.n_launches;
        }
        return check(c, "update_ghost_mr");
    }

    // Adapt::harten (mr/adapt.hpp:276-389) for one field
    int harten(Ctx& c, DeviceField& f, int ite, double eps, double regularity, bool* converged)
    {
        const Geom& g  = c.g;
        DeviceMesh& m  = c.m();
        const int minl = c.cfg.min_level;
        const int maxl = c.cfg.max_level;
        const int dim  = g.dim;
        int st;

        k_tag_init<<<grid_words(g.total_words), BLOCK, 0, c.stream>>>(g, m.ref, m.cells, c.tag, c.detail);
        ++c.n_launches;
        if ((st = check(c, "tag_init")))
        {
            return st;
        }
        if ((st = update_ghost_mr(c, f)))
        {
            return st;
        }

        const int dl0 = minl > 0 ? minl - 1 : 0;
        const int dl1 = maxl - ite - 1;
        if (dl1 >= dl0)
        {
            k_detail<<<grid_words(g.lv[dl1].woff + g.lv[dl1].nwords - g.lv[dl0].woff), BLOCK, 0, c.stream>>>(g, dl0, dl1, c.cfg.prediction_radius, m.ref,
                                                                                                              m.hc, m.hc2, f.data, c.detail);
            ++c.n_launches;
        }

        Eps e{};
        for (int l = minl; l <= maxl - ite; ++l)
        {
            const int exponent = dim * (maxl - l);
            e.eps[l]           = eps / (1 << exponent);
            e.fine[l]          = std::pow(2.0, regularity + dim) * e.eps[l];
            e.coarse[l]        = e.fine[l] / (1 << dim);
        }
        const int cl0 = minl, cl1 = maxl - ite;
        if (cl1 >= cl0 && cl0 >= 1)
        {
            k_criteria<<<grid_words(g.lv[cl1 - 1].woff + g.lv[cl1 - 1].nwords - g.lv[cl0 - 1].woff), BLOCK, 0, c.stream>>>(g, cl0, cl1, e, m.ref, m.hc,
                                                                                                                              c.detail, c.tag);
            ++c.n_launches;
        }
        for (int l = maxl; l > 0; --l)
        {
            k_maximum<<<grid_words(g.lv[l - 1].nwords), BLOCK, 0, c.stream>>>(g, l, m.ref, m.hc, c.tag);
            ++c.n_launches;
        }
        if ((st = check(c, "criteria")))
        {
            return st;
        }

        DeviceMesh& nm = c.spare();
        if ((st = new_cells_from_tags(c, m, nm.cells)))
        {
            return st;
        }
        if ((st = graduate(c, nm.cells, nullptr)))
        {
            return st;
        }
        bool same = false;
        if ((st = bitmaps_equal(c, nm.cells, m.cells, &same)))
        {
            return st;
        }
        if (same)
        {
            *converged = true;
            return SG_OK;
        }
        *converged = false;
        if ((st = build_mesh(c, nm)))
        {
            return st;
        }
        k_update_fields<<<grid_words(g.total_words), BLOCK, 0, c.stream>>>(g, c.cfg.prediction_radius, nm.ref, nm.cells, m.ref, m.cells, m.hc, f.data,
                                                                           f.spare);
        ++c.n_launches;
        if ((st = check(c, "update_fields")))
        {
            return st;
        }
        std::swap(f.data, f.spare);
        c.cur = 1 - c.cur;
        return SG_OK;
    }

    // Adapt::operator() (mr/adapt.hpp:147-195)
    int adapt(Ctx& c, DeviceField& f, double eps, double regularity, int* n_harten)
    {
        const int minl = c.cfg.min_level, maxl = c.cfg.max_level;
        int it         = 0;
        if (minl != maxl)
        {
            for (int i = 0; i < maxl - minl; ++i)
            {
                ++it;
                bool conv = false;
                int st    = harten(c, f, i, eps, regularity, &conv);
                if (st)
                {
                    return st;
                }
                if (conv)
                {
                    break;
                }
            }
        }
        if (n_harten)
        {
            *n_harten = it;
        }
        return device_error(c);
    }

    int upwind(Ctx& c, DeviceField& u, DeviceField& unp1, const double* a, double dt, int scheme)
    {
        const Geom& g = c.g;
        k_upwind<<<grid_words(g.total_words), BLOCK, 0, c.stream>>>(g, c.m().cells, u.data, unp1.data, a[0], a[1], g.dim == 3 ? a[2] : 0., dt, scheme);
        ++c.n_launches;
        return check(c, "upwind");
    }
} // namespace sg
