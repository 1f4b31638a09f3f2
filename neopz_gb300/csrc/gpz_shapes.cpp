// Host-side H1 shape tables and Gauss rules (see gpz_shapes.h).
#include "gpz_shapes.h"

#include <cmath>
#include <cstring>

#include "../../include/gpz.h"

namespace gpz {

namespace {

ElemTopo make_line() {
  ElemTopo t{};
  t.type = GPZ_EL_LINE;
  t.dim = 1;
  t.ncorner = 2;
  t.nsides = 3;
  double v[2][3] = {{-1, 0, 0}, {1, 0, 0}};
  std::memcpy(t.vert, v, sizeof(v));
  for (int s = 0; s < 2; s++) { t.side_dim[s] = 0; t.side_nnode[s] = 1; t.side_node[s][0] = s; }
  t.side_dim[2] = 1; t.side_nnode[2] = 2; t.side_node[2][0] = 0; t.side_node[2][1] = 1;
  return t;
}

ElemTopo make_quad() {
  ElemTopo t{};
  t.type = GPZ_EL_QUAD;
  t.dim = 2;
  t.ncorner = 4;
  t.nsides = 9;
  double v[4][3] = {{-1, -1, 0}, {1, -1, 0}, {1, 1, 0}, {-1, 1, 0}};
  std::memcpy(t.vert, v, sizeof(v));
  for (int s = 0; s < 4; s++) { t.side_dim[s] = 0; t.side_nnode[s] = 1; t.side_node[s][0] = s; }
  for (int s = 4; s < 8; s++) {
    t.side_dim[s] = 1; t.side_nnode[s] = 2;
    t.side_node[s][0] = s - 4; t.side_node[s][1] = (s - 3) % 4;
  }
  t.side_dim[8] = 2; t.side_nnode[8] = 4;
  for (int k = 0; k < 4; k++) t.side_node[8][k] = k;
  return t;
}

ElemTopo make_hex() {
  ElemTopo t{};
  t.type = GPZ_EL_HEX;
  t.dim = 3;
  t.ncorner = 8;
  t.nsides = 27;
  double v[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                    {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
  std::memcpy(t.vert, v, sizeof(v));
  const int edge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {0, 4}, {1, 5}, {2, 6}, {3, 7}, {4, 5}, {5, 6}, {6, 7}, {7, 4}};
  const int face[6][4] = {{0, 1, 2, 3}, {0, 1, 5, 4}, {1, 2, 6, 5}, {3, 2, 6, 7}, {0, 3, 7, 4}, {4, 5, 6, 7}};
  for (int s = 0; s < 8; s++) { t.side_dim[s] = 0; t.side_nnode[s] = 1; t.side_node[s][0] = s; }
  for (int e = 0; e < 12; e++) {
    t.side_dim[8 + e] = 1; t.side_nnode[8 + e] = 2;
    t.side_node[8 + e][0] = edge[e][0]; t.side_node[8 + e][1] = edge[e][1];
  }
  for (int f = 0; f < 6; f++) {
    t.side_dim[20 + f] = 2; t.side_nnode[20 + f] = 4;
    for (int k = 0; k < 4; k++) t.side_node[20 + f][k] = face[f][k];
  }
  t.side_dim[26] = 3; t.side_nnode[26] = 8;
  for (int k = 0; k < 8; k++) t.side_node[26][k] = k;
  return t;
}

const ElemTopo kLine = make_line(), kQuad = make_quad(), kHex = make_hex();

bool side_contains(const ElemTopo &t, int big, int small) {
  for (int i = 0; i < t.side_nnode[small]; i++) {
    bool found = false;
    for (int j = 0; j < t.side_nnode[big]; j++) found |= t.side_node[big][j] == t.side_node[small][i];
    if (!found) return false;
  }
  return true;
}

// TPZShapeQuad::gTrans2dQ: the eight orientations of a quadrilateral side
const double kQuadOrient[8][2][2] = {
    {{1., 0.}, {0., 1.}}, {{0., 1.}, {1., 0.}}, {{0., 1.}, {-1., 0.}}, {{-1., 0.}, {0., 1.}},
    {{-1., 0.}, {0., -1.}}, {{0., -1.}, {-1., 0.}}, {{0., -1.}, {1., 0.}}, {{1., 0.}, {0., -1.}}};

// Chebyshev T_0..T_{n-1} and derivatives
void cheb(double x, int n, double *p, double *d) {
  if (n <= 0) return;
  p[0] = 1.0; d[0] = 0.0;
  if (n == 1) return;
  p[1] = x; d[1] = 1.0;
  for (int k = 2; k < n; k++) {
    p[k] = 2.0 * x * p[k - 1] - p[k - 2];
    d[k] = 2.0 * x * d[k - 1] + 2.0 * p[k - 1] - d[k - 2];
  }
}

}  // namespace

const ElemTopo &topo(int type) { return type == GPZ_EL_LINE ? kLine : (type == GPZ_EL_QUAD ? kQuad : kHex); }

int side_nshape(int type, int s, int order) {
  int d = topo(type).side_dim[s];
  int m = order - 1;
  if (d == 0) return 1;
  if (m <= 0) return 0;
  return d == 1 ? m : (d == 2 ? m * m : m * m * m);
}

int side_orientation(int type, int s, const int64_t *ids) {
  const ElemTopo &t = topo(type);
  int d = t.side_dim[s];
  if (d == 1) return ids[t.side_node[s][0]] < ids[t.side_node[s][1]] ? 0 : 1;
  if (d == 2) {
    int64_t id[4];
    for (int k = 0; k < 4; k++) id[k] = ids[t.side_node[s][k]];
    int a = id[0] < id[1] ? 0 : 1, b = id[2] < id[3] ? 2 : 3;
    int mn = id[a] < id[b] ? a : b;
    int nxt = (mn + 1) % 4, prv = (mn + 3) % 4;
    int ccw = id[nxt] < id[prv];
    return 2 * mn + (ccw ? 0 : 1);
  }
  return 0;
}

int eval_shapes(int type, const int *orders, const int *trans, const double *pt, double *phi, double *dphi, int ld,
                int *side_of, int *k_of) {
  const ElemTopo &t = topo(type);
  const int D = t.dim, NC = t.ncorner, NS = t.nsides;
  // corner functions: product over the axes of (1 +/- x)/2
  double cphi[8], cd[3][8];
  for (int k = 0; k < NC; k++) {
    double f[3], g[3];
    for (int a = 0; a < D; a++) {
      double sgn = t.vert[k][a];
      f[a] = (1.0 + sgn * pt[a]) / 2.0;
      g[a] = sgn / 2.0;
    }
    double v = 1.0;
    for (int a = 0; a < D; a++) v *= f[a];
    cphi[k] = v;
    for (int a = 0; a < D; a++) {
      double dv = g[a];
      for (int b = 0; b < D; b++)
        if (b != a) dv *= f[b];
      cd[a][k] = dv;
    }
  }
  int n = 0;
  for (int k = 0; k < NC; k++) {
    phi[n] = cphi[k];
    for (int a = 0; a < D; a++) dphi[a * ld + n] = cd[a][k];
    if (side_of) { side_of[n] = k; k_of[n] = 0; }
    n++;
  }
  bool any = false;
  for (int s = NC; s < NS; s++) any |= side_nshape(type, s, orders[s - NC]) > 0;
  if (!any) return n;
  // raw blends: product of two corner functions (the side's first and its
  // opposite corner), then made unitary by adding every higher side's raw blend
  double raw[27], rawd[3][27];
  for (int s = NC; s < NS; s++) {
    int i0 = t.side_node[s][0];
    int i1 = t.side_dim[s] == 1 ? t.side_node[s][1] : t.side_node[s][2];
    if (t.side_dim[s] == 3) i1 = 6;
    raw[s] = cphi[i0] * cphi[i1];
    for (int a = 0; a < D; a++) rawd[a][s] = cd[a][i0] * cphi[i1] + cphi[i0] * cd[a][i1];
  }
  double bl[27], bld[3][27];
  for (int s = NC; s < NS; s++) {
    bl[s] = raw[s];
    for (int a = 0; a < D; a++) bld[a][s] = rawd[a][s];
    for (int h = s + 1; h < NS; h++) {
      if (t.side_dim[h] <= t.side_dim[s] || !side_contains(t, h, s)) continue;
      bl[s] += raw[h];
      for (int a = 0; a < D; a++) bld[a][s] += rawd[a][h];
    }
    double mult = t.side_dim[s] == 1 ? 4.0 : (t.side_dim[s] == 2 ? 16.0 : 64.0);
    bl[s] *= mult;
    for (int a = 0; a < D; a++) bld[a][s] *= mult;
  }
  for (int s = NC; s < NS; s++) {
    int ns = side_nshape(type, s, orders[s - NC]);
    if (ns == 0) continue;
    phi[n] = bl[s];
    for (int a = 0; a < D; a++) dphi[a * ld + n] = bld[a][s];
    if (side_of) { side_of[n] = s; k_of[n] = 0; }
    n++;
    if (ns == 1) continue;
    int sd = t.side_dim[s];
    // map element coordinates to side coordinates: M (sd x D)
    double M[3][3] = {{0}};
    if (sd == 3) {
      for (int a = 0; a < 3; a++) M[a][a] = 1.0;
    } else {
      double E[2][3] = {{0}};
      int v0 = t.side_node[s][0];
      int vv[2] = {t.side_node[s][1], sd == 2 ? t.side_node[s][3] : 0};
      for (int r = 0; r < sd; r++)
        for (int a = 0; a < D; a++) E[r][a] = (t.vert[vv[r]][a] - t.vert[v0][a]) / 2.0;
      double P[2][2] = {{1, 0}, {0, 1}};
      int o = trans[s - NC];
      if (sd == 1) P[0][0] = o ? -1.0 : 1.0;
      else
        for (int i = 0; i < 2; i++)
          for (int j = 0; j < 2; j++) P[i][j] = kQuadOrient[o][i][j];
      for (int i = 0; i < sd; i++)
        for (int a = 0; a < D; a++) {
          double acc = 0.0;
          for (int k = 0; k < sd; k++) acc += P[i][k] * E[k][a];
          M[i][a] = acc;
        }
    }
    double xs[3] = {0, 0, 0};
    for (int i = 0; i < sd; i++)
      for (int a = 0; a < D; a++) xs[i] += M[i][a] * pt[a];
    int m = orders[s - NC] - 1;
    double cp[3][8], cdv[3][8];
    for (int i = 0; i < sd; i++) cheb(xs[i], m, cp[i], cdv[i]);
    // tensor products in the reference's index order (last coordinate fastest)
    double pin[64], din[3][64];
    int cnt = 0;
    if (sd == 1) {
      for (int i = 0; i < m; i++, cnt++) { pin[cnt] = cp[0][i]; din[0][cnt] = cdv[0][i]; }
    } else if (sd == 2) {
      for (int i = 0; i < m; i++)
        for (int j = 0; j < m; j++, cnt++) {
          pin[cnt] = cp[0][i] * cp[1][j];
          din[0][cnt] = cdv[0][i] * cp[1][j];
          din[1][cnt] = cp[0][i] * cdv[1][j];
        }
    } else {
      for (int i = 0; i < m; i++)
        for (int j = 0; j < m; j++)
          for (int k = 0; k < m; k++, cnt++) {
            pin[cnt] = cp[0][i] * cp[1][j] * cp[2][k];
            din[0][cnt] = cdv[0][i] * cp[1][j] * cp[2][k];
            din[1][cnt] = cp[0][i] * cdv[1][j] * cp[2][k];
            din[2][cnt] = cp[0][i] * cp[1][j] * cdv[2][k];
          }
    }
    for (int i = 1; i < ns; i++) {
      phi[n] = bl[s] * pin[i];
      for (int a = 0; a < D; a++) {
        double g = 0.0;
        for (int k = 0; k < sd; k++) g += M[k][a] * din[k][i];
        dphi[a * ld + n] = bld[a][s] * pin[i] + bl[s] * g;
      }
      if (side_of) { side_of[n] = s; k_of[n] = i; }
      n++;
    }
  }
  return n;
}

void gauss_rule(int type, int order, std::vector<double> &pts, std::vector<double> &w) {
  int n = (int)(0.51 * (order + 2));
  if (n < 1) n = 1;
  // roots of P_n by Newton from the Tricomi-style initial guess, paired -z, +z
  std::vector<double> loc(n), wt(n);
  int m = (n + 1) / 2;
  for (int i = 0; i < m; i++) {
    long double z = std::cos(M_PI * (i + 0.75) / (n + 0.5)), dp = 0;
    for (int it = 0; it < 100; it++) {
      long double p0 = 1.0L, p1 = z;
      for (int k = 2; k <= n; k++) {
        long double pk = ((2.0L * k - 1.0L) * z * p1 - (k - 1.0L) * p0) / k;
        p0 = p1;
        p1 = pk;
      }
      if (n == 1) { p1 = z; p0 = 1.0L; }
      dp = n * (z * p1 - p0) / (z * z - 1.0L);
      long double dz = p1 / dp;
      z -= dz;
      if (std::fabs((double)dz) < 1e-19) break;
    }
    long double ww = 2.0L / ((1.0L - z * z) * dp * dp);
    loc[2 * i] = (double)(-z);
    wt[2 * i] = (double)ww;
    if (2 * i + 1 < n) { loc[2 * i + 1] = (double)z; wt[2 * i + 1] = (double)ww; }
  }
  pts.clear();
  w.clear();
  if (type == GPZ_EL_LINE) {
    for (int i = 0; i < n; i++) { pts.push_back(loc[i]); w.push_back(wt[i]); }
  } else if (type == GPZ_EL_QUAD) {
    for (int ip = 0; ip < n * n; ip++) {
      int ik = ip / n, ie = ip % n;
      pts.push_back(loc[ik]); pts.push_back(loc[ie]);
      w.push_back(wt[ik] * wt[ie]);
    }
  } else {
    for (int ip = 0; ip < n * n * n; ip++) {
      int ik = ip % n, ie = (ip / n) % n, iz = ip / (n * n);
      pts.push_back(loc[ik]); pts.push_back(loc[ie]); pts.push_back(loc[iz]);
      w.push_back(wt[ik] * wt[ie] * wt[iz]);
    }
  }
}

}  // namespace gpz
