// Host-side H1 shape tables and Gauss rules for the element buckets.
//
// The hierarchical H1 basis of TPZShapeH1<TSHAPE> (Shape/TPZShapeH1.cpp:41-116):
// corner (bi/tri)linear functions, one "blend" function per side made unitary
// (Shape/pzshapecube.cpp:93-152, Shape/pzshapequad.cpp:66-96,
// Shape/pzshapelinear.cpp:195-205) and, from order 3 on, blends times
// Chebyshev products (Shape/pzshapelinear.cpp:15-32) of the side coordinates
// after the orientation transform chosen from the corner node ids
// (Shape/pzgenericshape.cpp:12-68, Topology/tpzquadrilateral.cpp:591-618).
// Side coordinates are taken geometrically: along (v1 - v0)/2 and (v3 - v0)/2
// of the side's master-element vertices, which reproduces
// TPZCube/TPZQuadrilateral/TPZLine::TransformElementToSide.
#pragma once
#include <stdint.h>

#include <vector>

namespace gpz {

struct ElemTopo {
  int type, dim, ncorner, nsides;
  double vert[8][3];              // master coordinates of the corners
  int side_dim[27];
  int side_nnode[27];
  int side_node[27][8];           // corner ids of each side, in the reference's order
};

const ElemTopo &topo(int type);

// number of shape functions of side s at order p (NConnectShapeF)
int side_nshape(int type, int s, int order);

// orientation id of side s from the global corner ids (0/1 for ribs, 0..7 for faces)
int side_orientation(int type, int s, const int64_t *ids);

// Evaluate every shape at pt. orders/trans: one entry per non-corner side.
// dphi is [dim][ld]. Returns the number of shapes; side_of/k_of (optional)
// receive, per shape, its side and index inside the side.
int eval_shapes(int type, const int *orders, const int *trans, const double *pt, double *phi, double *dphi, int ld,
                int *side_of = nullptr, int *k_of = nullptr);

// Gauss-Legendre rule with npoints = int(0.51 (order + 2)) per direction, in
// the reference's interleaved order (-z0, +z0, -z1, ...), tensorised as
// TPZIntQuad (eta fastest) / TPZIntCube3D (ksi fastest).
void gauss_rule(int type, int order, std::vector<double> &pts, std::vector<double> &w);

}  // namespace gpz
