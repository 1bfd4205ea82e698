/* vti_oracle.c -- TEST INFRASTRUCTURE: the file output of the reference's
 * `fix lbm-psm-vti` restated in plain C, so that the repository's two VTI
 * writers (lbmpsm/host.py write_vti and host/lbmpsm_fix.cpp write_vti_files)
 * can be compared with it byte for byte.
 *
 * WriteVTI::execute_write_vti<T> (src/fix_LBM_PSM_writeVTI.h:82-253) on one
 * process (rank 0 of a 1 x 1 x 1 processor grid): the local piece covers the
 * interior nodes (iStart = jStart = kStart = 1, offsets 0); the fields are
 * cast from double to T (float or double) in node order, z outermost; the
 * piece is written as raw appended binary (a UInt32 byte count before each
 * array) or as ascii (ten values per line); then the .pvti master file.
 * Doubles and floats are formatted as std::ostream formats them by default
 * (six significant digits, the %g conversion).
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include "lbmpsm_oracle.h"

static void put_g(FILE* f, double v) { fprintf(f, "%g", v); }

/* local: the local array sizes with the halo (nxL, nyL, nzL; nzL = 1 in
 * 2-D); origin: the domain's boxlo (domain->boxlo, z ignored in 2-D); dx the
 * lattice spacing; solid, rho: one double per interior node, u: three per
 * node, as the field read computes them before the cast
 * (src/fix_LBM_PSM_writeVTI.h:153-169).  Returns 0, or -1 if a file cannot
 * be written. */
int orc_write_vti(const char* folder, const char* name, int timestep, int binary, int use_double,
                  int dimension, const int* local, const double* origin, double dx,
                  const double* solid, const double* rho, const double* u) {
  const int env = 1;
  const int nxL = local[0], nyL = local[1], nzL = dimension == 3 ? local[2] : 1;
  const int iStart = env, jStart = env, kStart = dimension == 3 ? env : 0;
  const int nx_i = nxL - env - iStart, ny_i = nyL - env - jStart;
  const int nz_i = dimension == 3 ? nzL - env - kStart : 1;
  const int offsetX = 0, offsetY = 0, offsetZ = 0;
  const int nxTot = nxL - 2 * env, nyTot = nyL - 2 * env, nzTot = dimension == 3 ? nzL - 2 * env : 1;
  const char* typeStr = use_double ? "Float64" : "Float32";
  const size_t scalarSize = use_double ? 8 : 4;
  const int nP = nx_i * ny_i * nz_i;
  char base[512], path[1024];
  snprintf(base, sizeof base, "%s.%08d", name, timestep);
  /* node coordinate of the first output node, LBMPSMLattice::initialise_domain
   * (src/LBM_PSM_lattice.cpp:162-164) on rank 0; then minus offset * dx */
  const double x1 = origin[0] + iStart * dx - dx * env + (0 - 0 * 2 * env) * dx;
  const double y1 = origin[1] + jStart * dx - dx * env + (0 - 0 * 2 * env) * dx;
  const double z1 = (dimension == 3 ? origin[2] : 0.0) + kStart * dx - dx * env + (0 - 0 * 2 * env) * dx;
  const double originX = x1 - offsetX * dx;
  const double originY = y1 - offsetY * dx;
  const double originZ = dimension == 3 ? z1 - offsetZ * dx : 0.0;
  /* the fields cast to T */
  void* B_o = malloc(scalarSize * (size_t)nP);
  void* rho_o = malloc(scalarSize * (size_t)nP);
  void* u_o = malloc(scalarSize * 3 * (size_t)nP);
  if (!B_o || !rho_o || !u_o) return -1;
  for (int id = 0; id < nP; ++id) {
    if (use_double) {
      ((double*)B_o)[id] = solid[id];
      ((double*)rho_o)[id] = rho[id];
      for (int c = 0; c < 3; ++c)
        ((double*)u_o)[3 * id + c] = c < 2 || dimension == 3 ? u[3 * id + c] : 0.0;
    } else {
      ((float*)B_o)[id] = (float)solid[id];
      ((float*)rho_o)[id] = (float)rho[id];
      for (int c = 0; c < 3; ++c)
        ((float*)u_o)[3 * id + c] = c < 2 || dimension == 3 ? (float)u[3 * id + c] : 0.0f;
    }
  }
  const int xE = offsetX + nx_i - 1, yE = offsetY + ny_i - 1;
  const int zE_ext = dimension == 3 ? offsetZ + nz_i - 1 : 0;
  snprintf(path, sizeof path, "%s/%s_rank0.vti", folder, base);
  FILE* f = fopen(path, binary ? "wb" : "w");
  if (!f) return -1;
  if (binary) {
    const uint32_t b_sz = (uint32_t)(nP * scalarSize);
    const uint32_t u_sz = (uint32_t)(nP * 3 * scalarSize);
    fprintf(f, "<?xml version=\"1.0\"?>\n<VTKFile type=\"ImageData\" version=\"1.0\" "
               "byte_order=\"LittleEndian\" header_type=\"UInt32\">\n");
    fprintf(f, " <ImageData WholeExtent=\"0 %d 0 %d 0 %d\" Origin=\"", nxTot - 1, nyTot - 1, nzTot - 1);
    put_g(f, originX); fputc(' ', f); put_g(f, originY); fputc(' ', f); put_g(f, originZ);
    fprintf(f, "\" Spacing=\"");
    put_g(f, dx); fputc(' ', f); put_g(f, dx); fputc(' ', f); put_g(f, dx);
    fprintf(f, "\">\n");
    fprintf(f, "  <Piece Extent=\"%d %d %d %d %d %d\">\n", offsetX, xE, offsetY, yE, offsetZ, zE_ext);
    fprintf(f, "   <PointData>\n");
    fprintf(f, "    <DataArray type=\"%s\" Name=\"SolidFraction\" format=\"appended\" offset=\"0\"/>\n", typeStr);
    fprintf(f, "    <DataArray type=\"%s\" Name=\"Density\" format=\"appended\" offset=\"%u\"/>\n",
            typeStr, (unsigned)(4 + b_sz));
    fprintf(f, "    <DataArray type=\"%s\" Name=\"Velocity\" NumberOfComponents=\"3\" format=\"appended\" "
               "offset=\"%u\"/>\n", typeStr, (unsigned)(2 * (4 + b_sz)));
    fprintf(f, "   </PointData>\n  </Piece>\n </ImageData>\n <AppendedData encoding=\"raw\">_");
    fwrite(&b_sz, 4, 1, f); fwrite(B_o, 1, b_sz, f);
    fwrite(&b_sz, 4, 1, f); fwrite(rho_o, 1, b_sz, f);
    fwrite(&u_sz, 4, 1, f); fwrite(u_o, 1, u_sz, f);
    fprintf(f, "\n </AppendedData>\n</VTKFile>");
  } else {
    fprintf(f, "<?xml version=\"1.0\"?>\n<VTKFile type=\"ImageData\" version=\"0.1\">\n");
    fprintf(f, " <ImageData WholeExtent=\"0 %d 0 %d 0 %d\" Origin=\"", nxTot - 1, nyTot - 1, nzTot - 1);
    put_g(f, originX); fputc(' ', f); put_g(f, originY); fputc(' ', f); put_g(f, originZ);
    fprintf(f, "\" Spacing=\"");
    put_g(f, dx); fputc(' ', f); put_g(f, dx); fputc(' ', f); put_g(f, dx);
    fprintf(f, "\">\n");
    fprintf(f, "  <Piece Extent=\"%d %d %d %d %d %d\">\n", offsetX, xE, offsetY, yE, offsetZ, zE_ext);
    fprintf(f, "   <PointData>\n");
    const char* names[3] = {"SolidFraction", "Density", "Velocity"};
    const int comps[3] = {1, 1, 3};
    const void* data[3] = {B_o, rho_o, u_o};
    for (int a = 0; a < 3; ++a) {
      fprintf(f, "    <DataArray type=\"%s\" Name=\"%s\" NumberOfComponents=\"%d\" format=\"ascii\">\n",
              typeStr, names[a], comps[a]);
      const size_t cnt = (size_t)nP * comps[a];
      for (size_t i = 0; i < cnt; ++i) {
        put_g(f, use_double ? ((const double*)data[a])[i] : (double)((const float*)data[a])[i]);
        fputc(i % 10 == 9 ? '\n' : ' ', f);
      }
      fprintf(f, "\n    </DataArray>\n");
    }
    fprintf(f, "   </PointData>\n  </Piece>\n </ImageData>\n</VTKFile>");
  }
  fclose(f);
  free(B_o);
  free(rho_o);
  free(u_o);
  snprintf(path, sizeof path, "%s/%s.pvti", folder, base);
  f = fopen(path, "w");
  if (!f) return -1;
  fprintf(f, "<?xml version=\"1.0\"?>\n<VTKFile type=\"PImageData\" version=\"0.1\">\n");
  fprintf(f, " <PImageData WholeExtent=\"0 %d 0 %d 0 %d\" Origin=\"", nxTot - 1, nyTot - 1, nzTot - 1);
  put_g(f, originX); fputc(' ', f); put_g(f, originY); fputc(' ', f); put_g(f, originZ);
  fprintf(f, "\" Spacing=\"");
  put_g(f, dx); fputc(' ', f); put_g(f, dx); fputc(' ', f); put_g(f, dx);
  fprintf(f, "\">\n");
  fprintf(f, "  <PPointData>\n");
  fprintf(f, "   <PDataArray type=\"%s\" Name=\"SolidFraction\"/>\n", typeStr);
  fprintf(f, "   <PDataArray type=\"%s\" Name=\"Density\"/>\n", typeStr);
  fprintf(f, "   <PDataArray type=\"%s\" Name=\"Velocity\" NumberOfComponents=\"3\"/>\n", typeStr);
  fprintf(f, "  </PPointData>\n");
  fprintf(f, "  <Piece Extent=\"%d %d %d %d %d %d\" Source=\"%s_rank0.vti\"/>\n", offsetX, xE, offsetY,
          yE, offsetZ, zE_ext, base);
  fprintf(f, " </PImageData>\n</VTKFile>");
  fclose(f);
  return 0;
}
