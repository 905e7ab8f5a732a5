// Host-side set-up: level geometry, element stiffness tables, cantilever load.
#include <cmath>
#include <cstring>
#include <vector>

#include "tp_internal.h"

namespace tp {

Level make_level(int nelx, int nely, int nelz, int l) {
  Level L;
  L.ex = nelx >> l;
  L.ey = nely >> l;
  L.ez = nelz >> l;
  L.nx = L.ex + 1;
  L.ny = L.ey + 1;
  L.nz = L.ez + 1;
  L.nnodes = (long)L.nx * L.ny * L.nz;
  L.ndof = 3 * L.nnodes;
  // two y-edge strips of nely_l/4 + 1 nodes across all z on the x=0 face
  // (stencil_grid_utility.c:34-59)
  L.lim = L.ey / 4 + 1;
  L.nfixed = 3L * L.nz * 2 * L.lim;
  return L;
}

// Element stiffness of each fine sub-cell of a level-l element, expressed in
// the level-l element's nodal DOFs: the integrals of getKEsubspace
// (local_matrix.c:251-319). That routine sums B^T C B over a 10-point
// midpoint rule per axis inside every sub-cell, with the iso eta coordinate
// flipped (local_matrix.c:297-298). Because the box Jacobian is diagonal and
// the rule is a tensor product, each entry factorises into products of 1-D
// sums of (shape function | derivative) x (shape function | derivative); this
// evaluates those 1-D sums and combines them for an isotropic C:
//   KE[(q,c),(p,d)] = a*h^3 * ( lambda*M(c,d) + mu*M(d,c) + [c==d] mu*sum_e M(e,e) ),
//   M(a,b)[q,p] = prod_dim S_dim[dim==a][dim==b][s_q,dim][s_p,dim],
// a = ncell/2 the element half size, h the quadrature spacing. It agrees
// with the reference's point-by-point sum to about 2e-15 relative.
void element_matrix_tables(double nu, int l, double* KE) {
  const int nc = 1 << l;
  const int ip = 10;
  const double a = 0.5 * nc;
  const double h = 2.0 / (double)nc / (double)ip;
  const double lambda = nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
  const double mu = 1.0 / (2.0 * (1.0 + nu));
  // iso signs of the 8 trilinear functions (xi, eta, zeta)
  static const int sg[3][8] = {{-1, 1, 1, -1, -1, 1, 1, -1},
                               {-1, -1, 1, 1, -1, -1, 1, 1},
                               {-1, -1, -1, -1, 1, 1, 1, 1}};
  for (int ii = 0; ii < nc; ii++)
    for (int kk = 0; kk < nc; kk++)
      for (int jj = 0; jj < nc; jj++) {
        double* K = KE + 576 * (nc * nc * ii + nc * kk + jj);
        // 1-D quadrature points per axis, accumulated as the reference does
        double pts[3][10];
        const int cell[3] = {ii, jj, kk};
        for (int dim = 0; dim < 3; dim++) {
          double g = -1.0 + h / 2.0 + 2.0 / (double)nc * ((double)cell[dim]);
          for (int t = 0; t < ip; t++) {
            pts[dim][t] = (dim == 1) ? -1.0 * g : g;
            g += h;
          }
        }
        // S[dim][da][db][s][t] = sum_p f_da(s, p) f_db(t, p)
        double S[3][2][2][2][2];
        for (int dim = 0; dim < 3; dim++)
          for (int da = 0; da < 2; da++)
            for (int db = 0; db < 2; db++)
              for (int s = 0; s < 2; s++)
                for (int t = 0; t < 2; t++) {
                  const double ss = s ? 1.0 : -1.0, ts = t ? 1.0 : -1.0;
                  double acc = 0.0;
                  for (int p = 0; p < ip; p++) {
                    const double x = pts[dim][p];
                    const double fa = da ? 0.5 * ss : 0.5 * (1.0 + ss * x);
                    const double fb = db ? 0.5 * ts : 0.5 * (1.0 + ts * x);
                    acc += fa * fb;
                  }
                  S[dim][da][db][s][t] = acc;
                }
        auto M = [&](int da, int db, int q, int p) {
          double v = 1.0;
          for (int dim = 0; dim < 3; dim++) {
            const int s = (sg[dim][q] + 1) / 2, t = (sg[dim][p] + 1) / 2;
            v *= S[dim][dim == da][dim == db][s][t];
          }
          return v;
        };
        const double scale = a * h * h * h;
        for (int q = 0; q < 8; q++)
          for (int p = 0; p < 8; p++)
            for (int c = 0; c < 3; c++)
              for (int d = 0; d < 3; d++) {
                double v = lambda * M(c, d, q, p) + mu * M(d, c, q, p);
                if (c == d) v += mu * (M(0, 0, q, p) + M(1, 1, q, p) + M(2, 2, q, p));
                K[24 * (3 * q + c) + 3 * p + d] = scale * v;
              }
      }
}

// -1 in z spread over the z=0 face nodes of the elements within ny/5 of
// (x = nelx, y = (nely-1)/2) (stencil_optimization.c:37-95).
void cantilever_load(const Level& L0, double* F) {
  const int nelx = L0.ex, nely = L0.ey;
  const int ny = L0.ny, nz = L0.nz;
  std::memset(F, 0, sizeof(double) * L0.ndof);
  const double radius = (double)ny / 5.0, r2 = radius * radius;
  const double cx = (double)nelx, cy = ((double)nely - 1.0) / 2.0;
  int cnt = 0;
  for (int i = 0; i < nelx; i++)
    for (int j = 0; j < nely; j++) {
      const double dx = i - cx, dy = j - cy;
      if (dx * dx + dy * dy < r2) cnt++;
    }
  const double f = -1.0 / (4.0 * (double)cnt);
  auto node = [&](int i, int j) { return ((long)i * nz + 0) * ny + j; };
  for (int i = 0; i < nelx; i++)
    for (int j = 0; j < nely; j++) {
      const double dx = i - cx, dy = j - cy;
      if (dx * dx + dy * dy < r2) {
        F[3 * node(i + 1, j + 1) + 2] += f;
        F[3 * node(i + 1, j) + 2] += f;
        F[3 * node(i, j + 1) + 2] += f;
        F[3 * node(i, j) + 2] += f;
      }
    }
}

}  // namespace tp
