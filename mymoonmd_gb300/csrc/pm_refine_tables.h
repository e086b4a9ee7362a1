// Refinement tables of the regular refinement of quadrilaterals, hexahedra
// and tetrahedra (child -> refined-cell vertex; the new vertices as the
// parent vertices they average), restated from the DatChildVertex /
// DatVertexChild / DatEdgeVertex arrays of src/Refinement/RefQuadRegDesc.C,
// RefHexaRegDesc.C and RefTetraRegDesc.C, and the Kuhn split of the unit cube
// of Default_UnitCube_Tetra (src/Geometry/Tests.C:1859-1912). Shared by the
// host refinement (pm_setup.cpp) and the device refinement (pm_devsetup.cu).
#pragma once

namespace pmsetup {

// refinement tables (child -> refined-cell vertex), restated from the
// DatChildVertex arrays of the regular refinement descriptors.
inline constexpr int kQuadChild[4][4] = {{0, 4, 8, 7}, {1, 5, 8, 4}, {2, 6, 8, 5}, {3, 7, 8, 6}};
// new quad vertices 4..8 as sets of parent vertices they average
inline constexpr int kQuadNew[5][4] = {{0, 1, -1, -1}, {1, 2, -1, -1}, {2, 3, -1, -1},
                                   {3, 0, -1, -1}, {0, 1, 2, 3}};

inline constexpr int kHexChild[8][8] = {
    {0, 8, 12, 11, 15, 16, 26, 24}, {1, 9, 12, 8, 13, 19, 26, 16},
    {2, 10, 12, 9, 17, 22, 26, 19}, {3, 11, 12, 10, 20, 24, 26, 22},
    {4, 23, 25, 14, 15, 24, 26, 16}, {5, 14, 25, 18, 13, 16, 26, 19},
    {6, 18, 25, 21, 17, 19, 26, 22}, {7, 21, 25, 23, 20, 22, 26, 24}};
// new hexa vertices 8..26: the children sharing them (DatVertexChild); child c
// carries parent vertex c, so the new vertex is the mean of those parent vertices
#define E -1, -1, -1, -1
inline constexpr int kHexNew[19][8] = {
    {0, 1, -1, -1, E}, {1, 2, -1, -1, E}, {2, 3, -1, -1, E}, {0, 3, -1, -1, E},
    {0, 1, 2, 3, E},   {1, 5, -1, -1, E}, {4, 5, -1, -1, E}, {0, 4, -1, -1, E},
    {0, 1, 4, 5, E},   {2, 6, -1, -1, E}, {5, 6, -1, -1, E}, {1, 2, 5, 6, E},
    {3, 7, -1, -1, E}, {6, 7, -1, -1, E}, {2, 3, 6, 7, E},   {4, 7, -1, -1, E},
    {0, 3, 4, 7, E},   {4, 5, 6, 7, E},   {0, 1, 2, 3, 4, 5, 6, 7}};
#undef E

inline constexpr int kTetChild[8][4] = {{0, 4, 6, 7}, {4, 1, 5, 8}, {6, 5, 2, 9}, {7, 8, 9, 3},
                                    {4, 6, 7, 8}, {5, 6, 4, 8}, {6, 7, 8, 9}, {8, 5, 6, 9}};
// new tetra vertices 4..9 are edge midpoints (DatEdgeVertex)
inline constexpr int kTetNew[6][2] = {{0, 1}, {1, 2}, {0, 2}, {0, 3}, {1, 3}, {2, 3}};

// Kuhn split of a cube into 6 tetrahedra, KVERT of Default_UnitCube_Tetra
// (src/Geometry/Tests.C:1859-1912), 0-based over the cube vertex numbering
// (0,0,0) (1,0,0) (1,1,0) (0,1,0) (0,0,1) (1,0,1) (1,1,1) (0,1,1).
inline constexpr int kKuhn[6][4] = {{0, 1, 2, 6}, {0, 5, 1, 6}, {0, 2, 3, 6},
                                {0, 3, 7, 6}, {0, 4, 5, 6}, {0, 7, 4, 6}};
inline constexpr int kCubeCorner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                      {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};

}  // namespace pmsetup
