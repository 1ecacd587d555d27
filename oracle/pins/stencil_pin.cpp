// Pins the oracle's 27-tap operator tables against the reference's own stencil
// algebra (src/general/stencil.h, compiled from the reference tree).
//
// It repeats the construction that InitDiscritizationStencil performs
// (src/pic/pic_field_solver_ecsim.cpp:7121-7310) for the d2E/dx^2 and
// d2E/dxdy stencils and prints every exported tap as JSON:
//   {"lap_x": [[i,j,k,a],...], "lap_y": ..., "lap_z": ..., "gd_xy": ..., "gd_xz": ..., "gd_yz": ...}
// Test infrastructure: the output is committed as tests/golden/stencil_taps.json.
#include <cstdio>

#include "stencil.h"

static void dump(const char* name, cStencil& s, bool last) {
  cStencil::cStencilData d;
  s.ExportStencil(&d);
  std::printf("\"%s\": [", name);
  for (int t = 0; t < d.Length; t++)
    std::printf("%s[%d,%d,%d,%.17g]", t ? "," : "", d.Data[t].i, d.Data[t].j, d.Data[t].k,
                d.Data[t].a);
  std::printf("]%s\n", last ? "" : ",");
}

int main() {
  // edge-centred averages of corner values (EdgeStencilPointTable rows 0, 4, 8)
  const int edge[3][6] = {{0, 0, -1, 0, -1, 0}, {-1, 0, 0, 0, -1, 0}, {-1, 0, -1, 0, 0, 0}};
  cStencil xEdge[3];
  for (int e = 0; e < 3; e++)
    for (int i = edge[e][0]; i <= edge[e][1]; i++)
      for (int j = edge[e][2]; j <= edge[e][3]; j++)
        for (int k = edge[e][4]; k <= edge[e][5]; k++) xEdge[e].add(0.25, i, j, k);

  cStencil face, lx, ly, lz;
  face.AddShifted(xEdge[0], 1, 0, 0);
  face.SubstractShifted(xEdge[0], 0, 0, 0, 2.0);
  face.AddShifted(xEdge[0], -1, 0, 0);
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 2; j++) lx.AddShifted(face, 0, i, j, 0.25);
  ly = lx;
  ly.SwitchAxes(0, 1);
  lz = lx;
  lz.SwitchAxes(0, 2);

  cStencil dy0 = xEdge[1], dz0 = xEdge[2];
  dy0.SubstractShifted(xEdge[1], 0, -1, 0);
  dz0.SubstractShifted(xEdge[2], 0, 0, -1);
  cStencil gxy, gxz, gyz;
  for (int l = 0; l < 2; l++)
    for (int m = 0; m < 2; m++) {
      gxy.AddShifted(dy0, 1, l, m, 0.25);
      gxy.SubstractShifted(dy0, 0, l, m, 0.25);
      gxz.AddShifted(dz0, 1, l, m, 0.25);
      gxz.SubstractShifted(dz0, 0, l, m, 0.25);
      gyz.AddShifted(dz0, l, 1, m, 0.25);
      gyz.SubstractShifted(dz0, l, 0, m, 0.25);
    }

  std::printf("{\n");
  dump("lap_x", lx, false);
  dump("lap_y", ly, false);
  dump("lap_z", lz, false);
  dump("gd_xy", gxy, false);
  dump("gd_xz", gxz, false);
  dump("gd_yz", gyz, true);
  std::printf("}\n");
  return 0;
}
