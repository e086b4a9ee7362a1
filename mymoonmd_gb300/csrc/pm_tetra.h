// Reference-tetrahedron data shared by the Stokes and the convection-diffusion
// assembly: the quadrature rules the reference picks for tetrahedra
// (TFEDatabase3D::QFTetraFromDegree, src/FE/FEDatabase3D.C:1003-1013:
// degree 3-4 -> P4Tetra, 5-6 -> P5Tetra; the rules of
// src/QuadFormulas/QuadFormulaTetra.C, points in the reference's order,
// weights summing to the volume 1/6) and the P1 / P2 Lagrange bases in local
// DOF order (include/FE3D/BF_C_T_P1_3D.h, BF_C_T_P2_3D.h).
#pragma once

namespace pm {

// P4Tetra (P4Exact): degree 4, 11 points (Keast's rule with a negative
// centroid weight)
inline constexpr int kP4n = 11;
inline constexpr double kP4w[11] = {-.0131555555555555555555555555556, .00762222222222222222222222222222,
                                    .00762222222222222222222222222222, .00762222222222222222222222222222,
                                    .00762222222222222222222222222222, .0248888888888888888888888888889,
                                    .0248888888888888888888888888889, .0248888888888888888888888888889,
                                    .0248888888888888888888888888889, .0248888888888888888888888888889,
                                    .0248888888888888888888888888889};
inline constexpr double kP4x[11] = {.25, .0714285714285714285714285714286, .785714285714285714285714285714,
                                    .0714285714285714285714285714286, .0714285714285714285714285714286,
                                    .399403576166799204996102147462, .399403576166799204996102147462,
                                    .100596423833200795003897852538, .100596423833200795003897852538,
                                    .100596423833200795003897852538, .399403576166799204996102147462};
inline constexpr double kP4y[11] = {.25, .0714285714285714285714285714286, .0714285714285714285714285714286,
                                    .785714285714285714285714285714, .0714285714285714285714285714286,
                                    .399403576166799204996102147462, .100596423833200795003897852538,
                                    .399403576166799204996102147462, .100596423833200795003897852538,
                                    .399403576166799204996102147462, .100596423833200795003897852538};
inline constexpr double kP4z[11] = {.25, .0714285714285714285714285714286, .0714285714285714285714285714286,
                                    .0714285714285714285714285714286, .785714285714285714285714285714,
                                    .100596423833200795003897852538, .399403576166799204996102147462,
                                    .399403576166799204996102147462, .399403576166799204996102147462,
                                    .100596423833200795003897852538, .100596423833200795003897852538};

// P5Tetra (P5Exact): degree 5, 15 points - the centroids of the four faces,
// the centroid of the cell, the four points (1/11, 1/11, 1/11, 8/11) and the
// six points (a, a, b, b) in barycentric coordinates
inline constexpr double kP5a = 0.066550153573664298239880464226303;
inline constexpr double kP5b = 0.43344984642633570176011953577370;
inline constexpr double kP5wf = 0.0060267857142857142857142857142857;  // face centroids (27/4480)
inline constexpr double kP5wc = 0.030283678097089175806376972557730;   // cell centroid
inline constexpr double kP5w11 = 0.011645249086028969410893609144338;  // (1/11, 1/11, 1/11, 8/11)
inline constexpr double kP5wab = 0.010949141561386459345643019112407;  // (a, a, b, b)
inline constexpr int kP5n = 15;
inline constexpr double kP5x[15] = {1.0 / 3, 1.0 / 3, 0.0, 1.0 / 3, 0.25, 1.0 / 11, 1.0 / 11, 8.0 / 11,
                                    1.0 / 11, kP5a, kP5b, kP5b, kP5a, kP5a, kP5b};
inline constexpr double kP5y[15] = {1.0 / 3, 0.0, 1.0 / 3, 1.0 / 3, 0.25, 1.0 / 11, 8.0 / 11, 1.0 / 11,
                                    1.0 / 11, kP5b, kP5a, kP5b, kP5a, kP5b, kP5a};
inline constexpr double kP5z[15] = {0.0, 1.0 / 3, 1.0 / 3, 1.0 / 3, 0.25, 8.0 / 11, 1.0 / 11, 1.0 / 11,
                                    1.0 / 11, kP5b, kP5b, kP5a, kP5b, kP5a, kP5a};
inline constexpr double kP5w[15] = {kP5wf,  kP5wf,  kP5wf,  kP5wf,  kP5wc,  kP5w11, kP5w11, kP5w11,
                                    kP5w11, kP5wab, kP5wab, kP5wab, kP5wab, kP5wab, kP5wab};

// C_T_P1_3D / C_T_P2_3D values and reference derivatives at (x, y, z)
inline void p1_eval(double x, double y, double z, double* v, double* dx, double* dy, double* dz) {
  v[0] = 1 - x - y - z;
  v[1] = x;
  v[2] = y;
  v[3] = z;
  const double gx[4] = {-1, 1, 0, 0}, gy[4] = {-1, 0, 1, 0}, gz[4] = {-1, 0, 0, 1};
  for (int i = 0; i < 4; ++i) {
    dx[i] = gx[i];
    dy[i] = gy[i];
    dz[i] = gz[i];
  }
}

inline void p2_eval(double x, double y, double z, double* v, double* dx, double* dy, double* dz) {
  v[0] = 1 - 3 * x - 3 * y - 3 * z + 2 * x * x + 4 * x * y + 4 * x * z + 2 * y * y + 4 * y * z + 2 * z * z;
  v[1] = 4 * x - 4 * x * x - 4 * x * y - 4 * x * z;
  v[2] = -x + 2 * x * x;
  v[3] = 4 * y - 4 * x * y - 4 * y * y - 4 * y * z;
  v[4] = 4 * x * y;
  v[5] = -y + 2 * y * y;
  v[6] = 4 * z - 4 * x * z - 4 * y * z - 4 * z * z;
  v[7] = 4 * x * z;
  v[8] = 4 * y * z;
  v[9] = -z + 2 * z * z;
  const double g0 = -3 + 4 * x + 4 * y + 4 * z;
  const double dxs[10] = {g0, 4 - 8 * x - 4 * y - 4 * z, -1 + 4 * x, -4 * y, 4 * y, 0, -4 * z, 4 * z, 0, 0};
  const double dys[10] = {g0, -4 * x, 0, 4 - 4 * x - 8 * y - 4 * z, 4 * x, -1 + 4 * y, -4 * z, 0, 4 * z, 0};
  const double dzs[10] = {g0, -4 * x, 0, -4 * y, 0, 0, 4 - 4 * x - 4 * y - 8 * z, 4 * x, 4 * y, -1 + 4 * z};
  for (int i = 0; i < 10; ++i) {
    dx[i] = dxs[i];
    dy[i] = dys[i];
    dz[i] = dzs[i];
  }
}

}  // namespace pm
