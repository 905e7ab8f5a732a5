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

// Level-l element matrices from moments. The coarse trilinear shape
// functions restricted to a sub-cell s are the sub-cell's own shape
// functions times the interpolation P_s, so the sub-cell tables above are
// exactly P_s^T KE0 P_s (same quadrature), and the element matrix is
// sum_s E_s P_s^T KE0 P_s. In the per-axis sum/difference basis
// (KE0 = T^T KZ T, KZ = T KE0 T^T / 64 with 45 non-zeros) one axis of P_s is
// [[1, 2m], [0, h]] -- m the sub-cell centre's offset from the element centre,
// h = 1/ncell, in element units -- so every entry of the element matrix is a
// fixed combination of the 27 moments
//   M[px*9 + py*3 + pz] = sum_s E_s mx^px my^py mz^pz,   p in {0,1,2}^3.
// For the block (li, lj) of local nodes and the entry q = 3c + d, the
// (moment, coefficient) pairs with a nonzero coefficient are listed in
// off[(li*8 + lj)*9 + q] .. off[... + 1]. The tables are checked against the
// sub-cell tables for random densities; false if they disagree.
bool moment_tables(const double* ke0, const double* ke_l, int l, std::vector<int>& off, std::vector<int>& pidx,
                   std::vector<double>& coef) {
  const int nc = 1 << l, nsub = nc * nc * nc;
  const double h = 1.0 / nc;
  auto loc = [](int dx, int dy, int dz) { return dz * 4 + (dy ? (dx ? 1 : 0) : (dx ? 2 : 3)); };
  double t8[8][8];
  for (int b = 0; b < 8; b++)
    for (int dx = 0; dx < 2; dx++)
      for (int dy = 0; dy < 2; dy++)
        for (int dz = 0; dz < 2; dz++) {
          const int bits[3] = {(b >> 2) & 1, (b >> 1) & 1, b & 1}, o[3] = {dx, dy, dz};
          double w = 1.0;
          for (int a = 0; a < 3; a++)
            if (bits[a]) w *= o[a] ? 1.0 : -1.0;
          t8[b][loc(dx, dy, dz)] = w;
        }
  std::vector<double> KZ(576, 0.0), G(576 * 27, 0.0), GE(576 * 27, 0.0);
  double kzmax = 0.0;
  for (int r = 0; r < 24; r++)
    for (int s = 0; s < 24; s++) {
      double acc = 0.0;
      for (int q = 0; q < 8; q++)
        for (int q2 = 0; q2 < 8; q2++) acc += t8[r / 3][q] * ke0[(3 * q + r % 3) * 24 + 3 * q2 + s % 3] * t8[s / 3][q2];
      KZ[r * 24 + s] = acc / 64.0;
      kzmax = std::fmax(kzmax, std::fabs(acc / 64.0));
    }
  for (int r = 0; r < 24; r++)
    for (int s = 0; s < 24; s++) {
      const double kz = KZ[r * 24 + s];
      if (std::fabs(kz) <= 1e-14 * kzmax) continue;
      const int b = r / 3, c = r % 3, b2 = s / 3, d = s % 3;
      for (int bp = 0; bp < 8; bp++) {
        if (b & ~bp) continue;
        for (int bq = 0; bq < 8; bq++) {
          if (b2 & ~bq) continue;
          double cf = kz;
          int p[3] = {0, 0, 0};
          for (int a = 0; a < 3; a++) {
            const int sh = 2 - a;  // bit of axis a (x, y, z)
            const int pr[2][2] = {{(b >> sh) & 1, (bp >> sh) & 1}, {(b2 >> sh) & 1, (bq >> sh) & 1}};
            for (int t = 0; t < 2; t++) {
              if (pr[t][0] == 0 && pr[t][1] == 1) {
                cf *= 2.0;
                p[a]++;
              } else if (pr[t][0] == 1) {
                cf *= h;
              }
            }
          }
          G[((3 * bp + c) * 24 + 3 * bq + d) * 27 + p[0] * 9 + p[1] * 3 + p[2]] += cf;
        }
      }
    }
  double gmax = 0.0;
  for (int i = 0; i < 8; i++)
    for (int j = 0; j < 8; j++)
      for (int c = 0; c < 3; c++)
        for (int d = 0; d < 3; d++)
          for (int p = 0; p < 27; p++) {
            double acc = 0.0;
            for (int bp = 0; bp < 8; bp++)
              for (int bq = 0; bq < 8; bq++) acc += t8[bp][i] * t8[bq][j] * G[((3 * bp + c) * 24 + 3 * bq + d) * 27 + p];
            GE[((3 * i + c) * 24 + 3 * j + d) * 27 + p] = acc;
            gmax = std::fmax(gmax, std::fabs(acc));
          }
  off.assign(64 * 9 + 1, 0);
  pidx.clear();
  coef.clear();
  for (int li = 0; li < 8; li++)
    for (int lj = 0; lj < 8; lj++)
      for (int q = 0; q < 9; q++) {
        const int c = q / 3, d = q % 3;
        off[(li * 8 + lj) * 9 + q] = (int)coef.size();
        for (int p = 0; p < 27; p++) {
          const double v = GE[((3 * li + c) * 24 + 3 * lj + d) * 27 + p];
          if (std::fabs(v) > 1e-13 * gmax) {
            pidx.push_back(p);
            coef.push_back(v);
          }
        }
      }
  off[64 * 9] = (int)coef.size();
  // check against sum_s E_s KE_s for pseudo-random densities in [1e-3, 1]
  std::vector<double> E(nsub), M(27, 0.0);
  unsigned long long st = 0x9e3779b97f4a7c15ULL + (unsigned)l;
  for (int s = 0; s < nsub; s++) {
    st = st * 6364136223846793005ULL + 1442695040888963407ULL;
    E[s] = 1e-3 + (1.0 - 1e-3) * (double)(st >> 11) * (1.0 / 9007199254740992.0);
  }
  for (int ii = 0; ii < nc; ii++)
    for (int kk = 0; kk < nc; kk++)
      for (int jj = 0; jj < nc; jj++) {
        const double m[3] = {(ii + 0.5) * h - 0.5, (jj + 0.5) * h - 0.5, (kk + 0.5) * h - 0.5};  // x, y, z
        const double e = E[(ii * nc + kk) * nc + jj];
        for (int p = 0; p < 27; p++) M[p] += e * std::pow(m[0], p / 9) * std::pow(m[1], (p / 3) % 3) * std::pow(m[2], p % 3);
      }
  double err = 0.0, ref = 0.0;
  for (int li = 0; li < 8; li++)
    for (int lj = 0; lj < 8; lj++)
      for (int q = 0; q < 9; q++) {
        const int r = 3 * li + q / 3, s = 3 * lj + q % 3;
        double direct = 0.0, mom = 0.0;
        for (int sb = 0; sb < nsub; sb++) direct += E[sb] * ke_l[(long)sb * 576 + r * 24 + s];
        const int b = (li * 8 + lj) * 9 + q;
        for (int k = off[b]; k < off[b + 1]; k++) mom += coef[k] * M[pidx[k]];
        err = std::fmax(err, std::fabs(mom - direct));
        ref = std::fmax(ref, std::fabs(direct));
      }
  return err <= 1e-12 * ref;
}

}  // namespace tp
