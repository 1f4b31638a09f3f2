// Grid meshes and their equation numbering (see pz_grid.h).
#include "pz_grid.h"

#include <algorithm>
#include <cstring>
#include <new>

namespace {

struct Grid {
  gpzh_grid_spec spec;
  int nstate = 1;
  int64_t nvol = 0;
  std::vector<double> xyz;
  // geometric elements: type, matid, corner nodes, side entities
  struct GEl {
    int type, matid;
    int64_t nodes[8];
    int64_t ent[27];
    int64_t cell;  // volume cell index or -1
  };
  std::vector<GEl> gels;
  int64_t nentities = 0;
  // computational mesh
  std::vector<int32_t> el_type, el_mat, el_order;
  std::vector<int64_t> el_nodes, el_conn;
  std::vector<double> el_coef;
  std::vector<int64_t> el_cell;              // grid cell of each element (-1: boundary element)
  std::vector<int32_t> conn_order, block_size;
  std::vector<int64_t> block_pos;
  int64_t neq = 0;
};

int nsides(int t) { return t == GPZ_EL_LINE ? 3 : (t == GPZ_EL_QUAD ? 9 : 27); }
int ncorner(int t) { return t == GPZ_EL_LINE ? 2 : (t == GPZ_EL_QUAD ? 4 : 8); }
int side_dim(int t, int s) {
  if (s < ncorner(t)) return 0;
  if (t == GPZ_EL_LINE) return 1;
  if (t == GPZ_EL_QUAD) return s < 8 ? 1 : 2;
  return s < 20 ? 1 : (s < 26 ? 2 : 3);
}
int nshape_of(int t, int s, int order) {
  int d = side_dim(t, s), m = order - 1;
  if (d == 0) return 1;
  if (m <= 0) return 0;
  return d == 1 ? m : (d == 2 ? m * m : m * m * m);
}

// Entity numbering of a structured grid.
struct Ent2 {
  int64_t nx, ny, nV, nEX, nEY, nC;
  int64_t V(int64_t i, int64_t j) const { return j * (nx + 1) + i; }
  int64_t EX(int64_t i, int64_t j) const { return nV + j * nx + i; }
  int64_t EY(int64_t i, int64_t j) const { return nV + nEX + j * (nx + 1) + i; }
  int64_t C(int64_t i, int64_t j) const { return nV + nEX + nEY + j * nx + i; }
  int64_t total() const { return nV + nEX + nEY + nC; }
};
struct Ent3 {
  int64_t nx, ny, nz;
  int64_t oEX, oEY, oEZ, oFXY, oFXZ, oFYZ, oC, tot;
  void init() {
    int64_t nV = (nx + 1) * (ny + 1) * (nz + 1);
    oEX = nV;
    oEY = oEX + nx * (ny + 1) * (nz + 1);
    oEZ = oEY + (nx + 1) * ny * (nz + 1);
    oFXY = oEZ + (nx + 1) * (ny + 1) * nz;
    oFXZ = oFXY + nx * ny * (nz + 1);
    oFYZ = oFXZ + nx * (ny + 1) * nz;
    oC = oFYZ + (nx + 1) * ny * nz;
    tot = oC + nx * ny * nz;
  }
  int64_t V(int64_t i, int64_t j, int64_t k) const { return (k * (ny + 1) + j) * (nx + 1) + i; }
  int64_t EX(int64_t i, int64_t j, int64_t k) const { return oEX + (k * (ny + 1) + j) * nx + i; }
  int64_t EY(int64_t i, int64_t j, int64_t k) const { return oEY + (k * ny + j) * (nx + 1) + i; }
  int64_t EZ(int64_t i, int64_t j, int64_t k) const { return oEZ + (k * (ny + 1) + j) * (nx + 1) + i; }
  int64_t FXY(int64_t i, int64_t j, int64_t k) const { return oFXY + (k * ny + j) * nx + i; }
  int64_t FXZ(int64_t i, int64_t j, int64_t k) const { return oFXZ + (k * (ny + 1) + j) * nx + i; }
  int64_t FYZ(int64_t i, int64_t j, int64_t k) const { return oFYZ + (k * ny + j) * (nx + 1) + i; }
  int64_t C(int64_t i, int64_t j, int64_t k) const { return oC + (k * ny + j) * nx + i; }
};

void build_1d(Grid &g) {
  const gpzh_grid_spec &s = g.spec;
  int64_t nx = s.ndiv[0];
  for (int64_t i = 0; i <= nx; i++) {
    g.xyz.push_back(s.minX[0] + ((s.maxX[0] - s.minX[0]) * i) / nx);
    g.xyz.push_back(0.0);
    g.xyz.push_back(0.0);
  }
  // entities: vertices 0..nx, segments nx+1..2nx
  for (int64_t i = 0; i < nx; i++) {
    Grid::GEl e{GPZ_EL_LINE, s.matids[0], {i, i + 1, -1, -1, -1, -1, -1, -1}, {}, i};
    e.ent[0] = i;
    e.ent[1] = i + 1;
    e.ent[2] = nx + 1 + i;
    g.gels.push_back(e);
  }
  g.nvol = nx;
  g.nentities = 2 * nx + 1;
}

// TPZGenGrid2D node / element / boundary order (Pre/TPZGenGrid2D.cpp:434-503,545-649,706-765)
void build_2d(Grid &g) {
  const gpzh_grid_spec &s = g.spec;
  Ent2 E;
  E.nx = s.ndiv[0];
  E.ny = s.ndiv[1];
  E.nV = (E.nx + 1) * (E.ny + 1);
  E.nEX = E.nx * (E.ny + 1);
  E.nEY = (E.nx + 1) * E.ny;
  E.nC = E.nx * E.ny;
  double dx = (s.maxX[0] - s.minX[0]) / E.nx, dy = (s.maxX[1] - s.minX[1]) / E.ny;
  for (int64_t j = 0; j <= E.ny; j++)
    for (int64_t i = 0; i <= E.nx; i++) {
      g.xyz.push_back(s.minX[0] + i * dx);
      g.xyz.push_back(s.minX[1] + j * dy);
      g.xyz.push_back(0.0);
    }
  for (int64_t j = 0; j < E.ny; j++)
    for (int64_t i = 0; i < E.nx; i++) {
      Grid::GEl e{};
      e.type = GPZ_EL_QUAD;
      e.matid = s.matids[0];
      e.cell = j * E.nx + i;
      int64_t v[4] = {E.V(i, j), E.V(i + 1, j), E.V(i + 1, j + 1), E.V(i, j + 1)};
      for (int k = 0; k < 4; k++) { e.nodes[k] = v[k]; e.ent[k] = v[k]; }
      for (int k = 4; k < 8; k++) e.nodes[k] = -1;
      e.ent[4] = E.EX(i, j);
      e.ent[5] = E.EY(i + 1, j);
      e.ent[6] = E.EX(i, j + 1);
      e.ent[7] = E.EY(i, j);
      e.ent[8] = E.C(i, j);
      g.gels.push_back(e);
    }
  g.nvol = E.nC;
  g.nentities = E.total();
  if (!s.create_bc) return;
  auto add_bc = [&](int matid, int64_t v0, int64_t v1, int64_t edge) {
    Grid::GEl e{};
    e.type = GPZ_EL_LINE;
    e.matid = matid;
    e.cell = -1;
    e.nodes[0] = v0; e.nodes[1] = v1;
    for (int k = 2; k < 8; k++) e.nodes[k] = -1;
    e.ent[0] = v0; e.ent[1] = v1; e.ent[2] = edge;
    g.gels.push_back(e);
  };
  for (int64_t i = 0; i < E.nx; i++) add_bc(s.matids[1], E.V(i, 0), E.V(i + 1, 0), E.EX(i, 0));             // side 4
  for (int64_t j = 0; j < E.ny; j++) add_bc(s.matids[2], E.V(E.nx, j), E.V(E.nx, j + 1), E.EY(E.nx, j));    // side 5
  for (int64_t i = 0; i < E.nx; i++) add_bc(s.matids[3], E.V(i + 1, E.ny), E.V(i, E.ny), E.EX(i, E.ny));    // side 6
  for (int64_t j = 0; j < E.ny; j++) add_bc(s.matids[4], E.V(0, j + 1), E.V(0, j), E.EY(0, j));            // side 7
}

// TPZGenGrid3D (Pre/TPZGenGrid3D.cpp:51-235 volume, 239-398 boundary)
void build_3d(Grid &g) {
  const gpzh_grid_spec &s = g.spec;
  Ent3 E;
  E.nx = s.ndiv[0];
  E.ny = s.ndiv[1];
  E.nz = s.ndiv[2];
  E.init();
  for (int64_t k = 0; k <= E.nz; k++)
    for (int64_t j = 0; j <= E.ny; j++)
      for (int64_t i = 0; i <= E.nx; i++) {
        g.xyz.push_back(s.minX[0] + ((s.maxX[0] - s.minX[0]) * i) / E.nx);
        g.xyz.push_back(s.minX[1] + ((s.maxX[1] - s.minX[1]) * j) / E.ny);
        g.xyz.push_back(s.minX[2] + ((s.maxX[2] - s.minX[2]) * k) / E.nz);
      }
  g.gels.reserve(E.nx * E.ny * E.nz + 2 * (E.nx * E.ny + E.ny * E.nz + E.nx * E.nz));
  for (int64_t k = 0; k < E.nz; k++)
    for (int64_t j = 0; j < E.ny; j++)
      for (int64_t i = 0; i < E.nx; i++) {
        Grid::GEl e{};
        e.type = GPZ_EL_HEX;
        e.matid = s.matids[0];
        e.cell = (k * E.ny + j) * E.nx + i;
        int64_t v[8] = {E.V(i, j, k),         E.V(i + 1, j, k),         E.V(i + 1, j + 1, k),
                        E.V(i, j + 1, k),     E.V(i, j, k + 1),         E.V(i + 1, j, k + 1),
                        E.V(i + 1, j + 1, k + 1), E.V(i, j + 1, k + 1)};
        for (int q = 0; q < 8; q++) { e.nodes[q] = v[q]; e.ent[q] = v[q]; }
        e.ent[8] = E.EX(i, j, k);
        e.ent[9] = E.EY(i + 1, j, k);
        e.ent[10] = E.EX(i, j + 1, k);
        e.ent[11] = E.EY(i, j, k);
        e.ent[12] = E.EZ(i, j, k);
        e.ent[13] = E.EZ(i + 1, j, k);
        e.ent[14] = E.EZ(i + 1, j + 1, k);
        e.ent[15] = E.EZ(i, j + 1, k);
        e.ent[16] = E.EX(i, j, k + 1);
        e.ent[17] = E.EY(i + 1, j, k + 1);
        e.ent[18] = E.EX(i, j + 1, k + 1);
        e.ent[19] = E.EY(i, j, k + 1);
        e.ent[20] = E.FXY(i, j, k);
        e.ent[21] = E.FXZ(i, j, k);
        e.ent[22] = E.FYZ(i + 1, j, k);
        e.ent[23] = E.FXZ(i, j + 1, k);
        e.ent[24] = E.FYZ(i, j, k);
        e.ent[25] = E.FXY(i, j, k + 1);
        e.ent[26] = E.C(i, j, k);
        g.gels.push_back(e);
      }
  g.nvol = E.nx * E.ny * E.nz;
  g.nentities = E.tot;
  if (!s.create_bc) return;
  auto add_bc = [&](int matid, const int64_t *v, const int64_t *edges, int64_t face) {
    Grid::GEl e{};
    e.type = GPZ_EL_QUAD;
    e.matid = matid;
    e.cell = -1;
    for (int q = 0; q < 4; q++) { e.nodes[q] = v[q]; e.ent[q] = v[q]; e.ent[4 + q] = edges[q]; }
    for (int q = 4; q < 8; q++) e.nodes[q] = -1;
    e.ent[8] = face;
    g.gels.push_back(e);
  };
  const int mZmin = s.matids[1], mXmin = s.matids[2], mYmin = s.matids[3], mXmax = s.matids[4], mYmax = s.matids[5],
            mZmax = s.matids[6];
  for (int64_t k = 0; k < E.nz + 1; k += E.nz)
    for (int64_t j = 0; j < E.ny; j++)
      for (int64_t i = 0; i < E.nx; i++) {
        int64_t v[4] = {E.V(i, j, k), E.V(i + 1, j, k), E.V(i + 1, j + 1, k), E.V(i, j + 1, k)};
        int64_t ed[4] = {E.EX(i, j, k), E.EY(i + 1, j, k), E.EX(i, j + 1, k), E.EY(i, j, k)};
        add_bc(k == 0 ? mZmin : mZmax, v, ed, E.FXY(i, j, k));
      }
  for (int64_t k = 0; k < E.nz; k++)
    for (int64_t j = 0; j < E.ny + 1; j += E.ny)
      for (int64_t i = 0; i < E.nx; i++) {
        int64_t v[4] = {E.V(i, j, k), E.V(i + 1, j, k), E.V(i + 1, j, k + 1), E.V(i, j, k + 1)};
        int64_t ed[4] = {E.EX(i, j, k), E.EZ(i + 1, j, k), E.EX(i, j, k + 1), E.EZ(i, j, k)};
        add_bc(j == 0 ? mYmin : mYmax, v, ed, E.FXZ(i, j, k));
      }
  for (int64_t k = 0; k < E.nz; k++)
    for (int64_t j = 0; j < E.ny; j++)
      for (int64_t i = 0; i < E.nx + 1; i += E.nx) {
        int64_t v[4] = {E.V(i, j, k), E.V(i, j + 1, k), E.V(i, j + 1, k + 1), E.V(i, j, k + 1)};
        int64_t ed[4] = {E.EY(i, j, k), E.EZ(i, j + 1, k), E.EY(i, j, k + 1), E.EZ(i, j, k)};
        add_bc(i == 0 ? mXmin : mXmax, v, ed, E.FYZ(i, j, k));
      }
}

int find_id(const int32_t *ids, int n, int id) {
  for (int i = 0; i < n; i++)
    if (ids[i] == id) return i;
  return -1;
}

// AutoBuild + InitializeBlock
void build_comp(Grid &g) {
  const gpzh_grid_spec &s = g.spec;
  g.nstate = 1;
  for (int i = 0; i < s.nmat; i++)
    if (s.mats[i].kind == GPZ_MAT_ELAST3D) g.nstate = 3;
  std::vector<int64_t> ent2conn(g.nentities, -1);
  // side order: max rule over the preferred orders of the volume elements on the side
  std::vector<int32_t> ent_order;
  if (s.elem_order) {
    ent_order.assign(g.nentities, 0);
    for (const auto &e : g.gels)
      if (e.cell >= 0 && find_id(s.mat_id, s.nmat, e.matid) >= 0)
        for (int q = 0; q < nsides(e.type); q++)
          ent_order[e.ent[q]] = std::max(ent_order[e.ent[q]], s.elem_order[e.cell]);
  }
  for (const auto &e : g.gels) {
    int im = find_id(s.mat_id, s.nmat, e.matid), ib = -1;
    if (im < 0) {
      ib = find_id(s.bc_id, s.nbc, e.matid);
      if (ib < 0) continue;  // no material object: no computational element
    }
    int ns = nsides(e.type);
    int pref = s.default_order;
    if (s.elem_order && e.cell >= 0) pref = s.elem_order[e.cell];
    g.el_type.push_back(e.type);
    g.el_mat.push_back(im >= 0 ? im : -(ib + 1));
    g.el_order.push_back(pref);
    for (int q = 0; q < 8; q++) g.el_nodes.push_back(e.nodes[q]);
    for (int q = 0; q < 27; q++) {
      if (q >= ns) {
        g.el_conn.push_back(0);  // padding, rewritten below
        continue;
      }
      int64_t ent = e.ent[q];
      if (ent2conn[ent] < 0) {
        ent2conn[ent] = (int64_t)g.conn_order.size();
        int d = side_dim(e.type, q);
        int order = d == 0 ? 1 : (s.elem_order ? ent_order[ent] : s.default_order);
        g.conn_order.push_back(order);
        g.block_size.push_back(nshape_of(e.type, q, order) * g.nstate);
      }
      g.el_conn.push_back(ent2conn[ent]);
    }
    g.el_coef.push_back(s.elem_coef && e.cell >= 0 ? s.elem_coef[e.cell] : 0.0);
    g.el_cell.push_back(e.cell >= 0 ? e.cell : -1);
  }
  // fix the padding: unused slots repeat connect 0 (never read)
  for (size_t e = 0; e < g.el_type.size(); e++)
    for (int q = nsides(g.el_type[e]); q < 27; q++) g.el_conn[e * 27 + q] = g.el_conn[e * 27];
  g.block_pos.resize(g.conn_order.size());
  int64_t pos = 0;
  for (size_t i = 0; i < g.conn_order.size(); i++) {
    g.block_pos[i] = pos;
    pos += g.block_size[i];
  }
  g.neq = pos;
}

}  // namespace

extern "C" {

void *gpzh_grid_build(const gpzh_grid_spec *spec) {
  if (!spec) return nullptr;
  Grid *g = new (std::nothrow) Grid();
  if (!g) return nullptr;
  g->spec = *spec;
  if (spec->dim == 1) build_1d(*g);
  else if (spec->dim == 2) build_2d(*g);
  else build_3d(*g);
  build_comp(*g);
  g->spec.elem_coef = nullptr;
  g->spec.elem_order = nullptr;
  return g;
}

void gpzh_grid_free(void *grid) { delete (Grid *)grid; }

int gpzh_grid_desc(void *grid, gpz_mesh_desc *d) {
  Grid *g = (Grid *)grid;
  if (!g || !d) return GPZ_E_INVALID;
  std::memset(d, 0, sizeof(*d));
  d->dim = g->spec.dim;
  d->nstate = g->nstate;
  d->nnodes = (int64_t)g->xyz.size() / 3;
  d->node_xyz = g->xyz.data();
  d->nel = (int64_t)g->el_type.size();
  d->el_type = g->el_type.data();
  d->el_mat = g->el_mat.data();
  d->el_nodes = g->el_nodes.data();
  d->el_order = g->el_order.data();
  d->el_conn = g->el_conn.data();
  bool anycoef = false;
  for (double v : g->el_coef) anycoef |= v != 0.0;
  d->el_coef = anycoef ? g->el_coef.data() : nullptr;
  d->nconnects = (int64_t)g->conn_order.size();
  d->conn_order = g->conn_order.data();
  d->block_pos = g->block_pos.data();
  d->block_size = g->block_size.data();
  d->neq = g->neq;
  d->nmat = g->spec.nmat;
  d->mats = g->spec.mats;
  d->nbc = g->spec.nbc;
  d->bcs = g->spec.bcs;
  return GPZ_OK;
}

int64_t gpzh_grid_neq(void *grid) { return grid ? ((Grid *)grid)->neq : -1; }
int64_t gpzh_grid_nel(void *grid) { return grid ? (int64_t)((Grid *)grid)->el_type.size() : -1; }
int64_t gpzh_grid_nvol(void *grid) { return grid ? ((Grid *)grid)->nvol : -1; }

int gpzh_grid_cells(void *grid, int64_t *cell) {
  Grid *g = (Grid *)grid;
  if (!g || !cell) return -1;
  for (size_t e = 0; e < g->el_cell.size(); e++) cell[e] = g->el_cell[e];
  return 0;
}

int gpzh_grid_dest(void *grid, int64_t e, int64_t *dest) {
  Grid *g = (Grid *)grid;
  if (!g || e < 0 || e >= (int64_t)g->el_type.size()) return -1;
  int n = 0;
  for (int q = 0; q < nsides(g->el_type[e]); q++) {
    int64_t c = g->el_conn[e * 27 + q];
    for (int k = 0; k < g->block_size[c]; k++) dest[n++] = g->block_pos[c] + k;
  }
  return n;
}

}  // extern "C"
