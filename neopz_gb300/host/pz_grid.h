// Host-side computational mesh for grid domains, as the reference builds it
// with TPZGeoMeshTools::CreateGeoMeshOnGrid (Mesh/TPZGeoMeshTools.cpp:104-206)
// followed by TPZCompMesh::AutoBuild (Mesh/pzcmesh.cpp:393-409) and
// TPZCompMesh::InitializeBlock: geometric nodes and elements in the
// generator's order (volume elements first, then the boundary elements of
// TPZGenGrid2D::SetBC / TPZGenGrid3D::BuildBoundaryElements), computational
// elements in geometric-element order, and one connect per element side,
// numbered by first use (TPZInterpolatedElement::CreateMidSideConnect,
// Mesh/pzintel.cpp:652-730).  The numbering is computed from the grid's
// entities (vertices, x/y/z edges, faces, cells) instead of neighbour searches.
#pragma once
#include <stdint.h>

#include <vector>

#include "gpz.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int32_t dim;            /* 1, 2 or 3 */
  int32_t ndiv[3];
  double minX[3], maxX[3];
  int32_t matids[7];      /* 2D: {vol, bottom, right, top, left}; 3D: {vol, zmin, xmin, ymin, xmax, ymax, zmax} */
  int32_t create_bc;
  int32_t default_order;  /* TPZCompMesh::SetDefaultOrder */
  int32_t nmat;
  int32_t mat_id[4];      /* material id of mats[i] (InsertMaterialObject) */
  gpz_material mats[4];
  int32_t nbc;
  int32_t bc_id[8];       /* material id of bcs[i] */
  gpz_bc bcs[8];
  const double *elem_coef;  /* per volume element coefficient (cell index order) or NULL */
  const int32_t *elem_order;/* per volume element preferred order (hp) or NULL */
} gpzh_grid_spec;

void *gpzh_grid_build(const gpzh_grid_spec *spec);
void gpzh_grid_free(void *grid);
int gpzh_grid_desc(void *grid, gpz_mesh_desc *out);
int64_t gpzh_grid_neq(void *grid);
int64_t gpzh_grid_nel(void *grid);
int64_t gpzh_grid_nvol(void *grid);
/* grid cell index of every element (-1 for boundary elements), nel entries */
int gpzh_grid_cells(void *grid, int64_t *cell);
/* destination equations of computational element e (TPZElementMatrix::ComputeDestinationIndices) */
int gpzh_grid_dest(void *grid, int64_t e, int64_t *dest);

#ifdef __cplusplus
}
#endif
