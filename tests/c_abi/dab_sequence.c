/*
 * A C caller of libsculptgpu's C ABI (include/sculpt_gpu.h), compiled as C99:
 * the call sequence a reference-side sculpt stroke makes per dab —
 * BKE_pbvh_search_gather with the sphere callback, do_draw_brush on the
 * gathered nodes for each symmetry pass, BKE_pbvh_update_normals,
 * BKE_pbvh_update_bounds(UpdateBB) — then UpdateOriginalBB at the stroke end.
 *
 * usage: dab_sequence <mesh.bin> <dabs.bin> <out.bin>
 *   mesh.bin: int32 totvert, totpoly, totloop, totlt, leaf_limit, then the
 *             SGPU_MVert, SGPU_MPoly, SGPU_MLoop and SGPU_MLoopTri arrays
 *   dabs.bin: int32 ndabs, symmetry; float radius, strength; then ndabs
 *             SGPU_Dab
 *   out.bin:  the vertices (SGPU_MVert) and normals (3 floats) after the
 *             stroke, then the node boxes (vb, orig_vb; 6 floats per node)
 * Exit status 0 on success; the library's error text on stderr otherwise.
 */
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "sculpt_gpu.h"

/* The element layouts must be the reference's (types_meshdata.h:13-181). */
_Static_assert(sizeof(SGPU_MVert) == 16, "MVert is 16 bytes");
_Static_assert(offsetof(SGPU_MVert, flag) == 12 && offsetof(SGPU_MVert, bweight) == 13,
               "MVert flag/bweight follow co");
_Static_assert(sizeof(SGPU_MPoly) == 12, "MPoly is 12 bytes");
_Static_assert(offsetof(SGPU_MPoly, totloop) == 4 && offsetof(SGPU_MPoly, mat_nr) == 8 &&
                   offsetof(SGPU_MPoly, flag) == 10,
               "MPoly field offsets");
_Static_assert(sizeof(SGPU_MLoop) == 8 && offsetof(SGPU_MLoop, e) == 4, "MLoop layout");
_Static_assert(sizeof(SGPU_MLoopTri) == 16 && offsetof(SGPU_MLoopTri, poly) == 12,
               "MLoopTri layout");
_Static_assert(sizeof(SGPU_Dab) == 24, "a dab is six floats");

static int fail(const char *what, int rc)
{
  fprintf(stderr, "%s failed (%d): %s\n", what, rc, sgpu_last_error());
  return 1;
}

static void *read_all(FILE *f, size_t bytes)
{
  void *p = malloc(bytes > 0 ? bytes : 1);
  if (p && bytes > 0 && fread(p, 1, bytes, f) != bytes) {
    free(p);
    return NULL;
  }
  return p;
}

int main(int argc, char **argv)
{
  if (argc != 4) {
    fprintf(stderr, "usage: %s mesh.bin dabs.bin out.bin\n", argv[0]);
    return 2;
  }
  FILE *fm = fopen(argv[1], "rb"), *fd = fopen(argv[2], "rb");
  if (!fm || !fd) {
    fprintf(stderr, "cannot open the input files\n");
    return 2;
  }
  int head[5];
  if (fread(head, sizeof(int), 5, fm) != 5) {
    return 2;
  }
  const int totvert = head[0], totpoly = head[1], totloop = head[2], totlt = head[3];
  SGPU_MVert *verts = read_all(fm, sizeof(SGPU_MVert) * (size_t)totvert);
  SGPU_MPoly *polys = read_all(fm, sizeof(SGPU_MPoly) * (size_t)totpoly);
  SGPU_MLoop *loops = read_all(fm, sizeof(SGPU_MLoop) * (size_t)totloop);
  SGPU_MLoopTri *lts = read_all(fm, sizeof(SGPU_MLoopTri) * (size_t)totlt);
  int dh[2];
  float dp[2];
  if (!verts || !polys || !loops || !lts || fread(dh, sizeof(int), 2, fd) != 2 ||
      fread(dp, sizeof(float), 2, fd) != 2) {
    fprintf(stderr, "short input\n");
    return 2;
  }
  const int ndabs = dh[0], symmetry = dh[1];
  SGPU_Dab *dabs = read_all(fd, sizeof(SGPU_Dab) * (size_t)ndabs);
  if (!dabs) {
    return 2;
  }
  fclose(fm);
  fclose(fd);

  /* BKE_pbvh_new + BKE_pbvh_build_mesh */
  sgpu_mesh *mesh = NULL;
  int rc = sgpu_mesh_create_faces(verts, totvert, polys, totpoly, loops, totloop, lts, totlt,
                                  NULL, NULL, NULL, head[4], &mesh);
  if (rc) {
    return fail("sgpu_mesh_create_faces", rc);
  }
  SGPU_MeshInfo info;
  if ((rc = sgpu_mesh_info(mesh, &info))) {
    return fail("sgpu_mesh_info", rc);
  }
  SGPU_Brush brush;
  memset(&brush, 0, sizeof(brush));
  brush.sculpt_tool = SGPU_TOOL_DRAW;
  brush.symmetry = symmetry;
  brush.curve_preset = SGPU_CURVE_PRESET_SMOOTH;
  brush.radius = dp[0];
  brush.strength = dp[1];
  brush.normal_radius_factor = 0.5f;
  brush.area_radius_factor = 0.5f;
  brush.view_normal[2] = 1.0f;
  brush.crease_pinch_factor = 0.5f;
  brush.elastic_deform_volume_preservation = 0.4f;
  const float radius_sq = brush.radius * brush.radius;
  int *nodes = malloc(sizeof(int) * (size_t)(info.totleaf > 0 ? info.totleaf : 1));
  for (int d = 0; d < ndabs; d++) {
    for (int pass = 0; pass < 8; pass++) {
      if ((pass & ~symmetry) != 0) {
        continue;
      }
      float loc[3], delta[3];
      for (int k = 0; k < 3; k++) {
        const float sgn = (pass & (1 << k)) ? -1.0f : 1.0f;
        loc[k] = sgn * dabs[d].location[k];
        delta[k] = sgn * dabs[d].grab_delta[k];
      }
      /* BKE_pbvh_search_gather with the sphere callback */
      int tot = 0;
      if ((rc = sgpu_search_sphere(mesh, loc, radius_sq, 0, nodes, &tot))) {
        return fail("sgpu_search_sphere", rc);
      }
      if (tot == 0) {
        continue;
      }
      /* do_draw_brush(sd, ob, nodes, totnode) */
      if ((rc = sgpu_do_draw_brush(mesh, &brush, loc, delta, nodes, tot))) {
        return fail("sgpu_do_draw_brush", rc);
      }
    }
    if ((rc = sgpu_pbvh_update_normals(mesh))) {
      return fail("sgpu_pbvh_update_normals", rc);
    }
    if ((rc = sgpu_pbvh_update_bounds(mesh, SGPU_PBVH_UpdateBB))) {
      return fail("sgpu_pbvh_update_bounds", rc);
    }
  }
  if ((rc = sgpu_pbvh_update_bounds(mesh, SGPU_PBVH_UpdateOriginalBB))) {
    return fail("sgpu_pbvh_update_bounds", rc);
  }
  SGPU_MVert *out = malloc(sizeof(SGPU_MVert) * (size_t)totvert);
  float *no = malloc(sizeof(float) * 3 * (size_t)totvert);
  float *vb = malloc(sizeof(float) * 6 * (size_t)info.totnode);
  float *ovb = malloc(sizeof(float) * 6 * (size_t)info.totnode);
  if ((rc = sgpu_get_verts(mesh, out)) || (rc = sgpu_get_normals(mesh, no)) ||
      (rc = sgpu_get_node_bbs(mesh, vb, ovb))) {
    return fail("sgpu_get_*", rc);
  }
  FILE *fo = fopen(argv[3], "wb");
  if (!fo) {
    return 2;
  }
  fwrite(out, sizeof(SGPU_MVert), (size_t)totvert, fo);
  fwrite(no, sizeof(float), 3 * (size_t)totvert, fo);
  fwrite(vb, sizeof(float), 6 * (size_t)info.totnode, fo);
  fwrite(ovb, sizeof(float), 6 * (size_t)info.totnode, fo);
  fclose(fo);
  if ((rc = sgpu_mesh_destroy(mesh))) {
    return fail("sgpu_mesh_destroy", rc);
  }
  free(verts);
  free(polys);
  free(loops);
  free(lts);
  free(dabs);
  free(nodes);
  free(out);
  free(no);
  free(vb);
  free(ovb);
  return 0;
}
