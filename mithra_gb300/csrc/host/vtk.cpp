// Field visualization files: the XML structured-grid (.vts) and parallel index (.pvts) files of
// FdTd::fieldVisualizeAllDomain and fieldVisualizeInPlane{X,Y,Z}Normal (src/fdtd.cpp:956-1540;
// FdTdSC adds the scalar potential, src/fdtdSC.cpp:1263-1920), written on the host from E, B, A^n
// (and phi^n) downloaded from the device.
//
// The text is the reference's, value for value: scientific notation with four decimals, one
// node per line, nodes in the reference's order, the same header strings (including their
// irregular spacing), and the same coordinates, which for the y- and z-normal planes interpolate
// the x coordinate with the plane's fraction (as the reference does) while y and z come from the
// lower node.  Only interior nodes (1 .. N-2 transversally) carry values; the others are written
// as zero, the value the reference's buffers hold there.  One domain: the single piece spans the
// whole mesh (rank 0 of 1).
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "../../../include/mithra_gpu.h"

namespace {

struct Out {
  FILE* f = nullptr;
  explicit Out(const std::string& path) : f(std::fopen(path.c_str(), "w")) {}
  ~Out() {
    if (f) std::fclose(f);
  }
  void line(const char* s) { std::fprintf(f, "%s\n", s); }
};

// The node value of field code `c` (Seed::fieldType order: Ex Ey Ez Bx By Bz Ax Ay Az F).
double value(int c, long long m, const float* en, const float* bn, const double* an, const double* fn) {
  if (c < 3) return (double)en[3 * m + c];
  if (c < 6) return (double)bn[3 * m + c - 3];
  if (c < 9) return an[3 * m + c - 6];
  return fn ? fn[m] : 0.0;  // FdTd has no scalar potential: its buffer stays zero
}

void header(Out& o, const char* whole, const char* piece) {
  o.line("<?xml version=\"1.0\"?>");
  o.line("<VTKFile type=\"StructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\" compressor=\"vtkZLibDataCompressor\">");
  o.line(whole);
  o.line(piece);
  o.line("<Points>");
  o.line("<DataArray type = \"Float64\" NumberOfComponents=\"3\" format=\"ascii\">");
}

void middle(Out& o, int nfield) {
  o.line("</DataArray>");
  o.line("</Points>");
  o.line("<CellData>");
  o.line("</CellData>");
  o.line("<PointData Vectors = \"field\">");
  std::fprintf(o.f, "<DataArray type=\"Float64\" Name=\"field\" NumberOfComponents=\"%d\" format=\"ascii\">\n", nfield);
}

void footer(Out& o) {
  o.line("</DataArray>");
  o.line("</PointData>");
  o.line("</Piece>");
  o.line("</StructuredGrid>");
  o.line("</VTKFile>");
}

void values_line(Out& o, const double* v, int nfield) {
  std::fprintf(o.f, "%.4e", v[0]);
  for (int l = 1; l < nfield; l++) std::fprintf(o.f, " %.4e", v[l]);
  std::fputc('\n', o.f);
}

void pvts(const std::string& path, const char* whole, const char* piece_fmt, int nfield, const std::string& source) {
  Out o(path);
  o.line("<?xml version=\"1.0\"?>");
  o.line("<VTKFile type=\"PStructuredGrid\" version=\"0.1\" >");
  o.line(whole);
  o.line("<PPoints>");
  o.line("<DataArray type = \"Float64\" NumberOfComponents=\"3\" format=\"ascii\" />");
  o.line("</PPoints>");
  o.line("<PPointData>");
  std::fprintf(o.f, "<DataArray type=\"Float64\" NumberOfComponents=\"%d\" Name=\"field\" format=\"ascii\" />\n", nfield);
  o.line("</PPointData>");
  std::fprintf(o.f, piece_fmt, source.c_str());
  o.line("</PStructuredGrid>");
  o.line("</VTKFile>");
}

}  // namespace

extern "C" int mithra_vtk_write_field(const mithra_vtk_desc* d, const char* basename, long long n_time,
                                      const float* en, const float* bn, const double* an, const double* fn) {
  if (!d || !basename || !en || !bn || !an || d->nfield < 1 || d->nfield > MITHRA_VTK_MAX_FIELDS) return MITHRA_ERR_ARG;
  const int N0 = d->N0, N1 = d->N1, N2 = d->N2, np = d->np, k0 = d->k0, nf = d->nfield;
  const long long N1N0 = (long long)N1 * N0;
  const std::string base(basename);
  const std::string name = base.substr(base.find_last_of('/') + 1);
  const std::string tag = std::to_string(n_time);
  const std::string vts = base + "-p0-" + tag + ".vts", source = name + "-p0-" + tag + ".vts";
  const std::string pv = base + "-" + tag + ".pvts";
  // Solver::rc (src/solver.cpp:2302-2315)
  auto rx = [&](long long m) { return d->xmin + (double)(unsigned)((m % N1N0) / N1) * d->dx; };
  auto ry = [&](long long m) { return d->ymin + (double)(unsigned)(m - N1N0 * (m / N1N0) - N1 * ((m % N1N0) / N1)) * d->dy; };
  auto rz = [&](long long m) { return d->zmin + (double)(unsigned)(m / N1N0 + k0) * d->dz; };
  char whole[256], piece[256];
  double v[MITHRA_VTK_MAX_FIELDS];
  const int k_last = k0 + np - 1;  // k0 + np - 2 + 1 on the last (only) rank

  if (d->type == 0) {  // all-domain, src/fdtd.cpp:956-1106
    std::vector<double> vals((size_t)N1N0 * np * nf, 0.0);
    for (int k = 0; k < np; k++)
      for (int j = 1; j < N1 - 1; j++)
        for (int i = 1; i < N0 - 1; i++) {
          const long long m = k * N1N0 + (long long)i * N1 + j;
          for (int l = 0; l < nf; l++) vals[(size_t)m * nf + l] = value(d->field[l], m, en, bn, an, fn);
        }
    {
      Out o(vts);
      if (!o.f) return MITHRA_ERR_ARG;
      std::snprintf(whole, sizeof whole, "<StructuredGrid WholeExtent=\"0 %d 0 %d %d %d\">", N0 - 1, N1 - 1, k0, k_last);
      std::snprintf(piece, sizeof piece, "<Piece Extent=\"0 %d 0 %d %d %d\">", N0 - 1, N1 - 1, k0, k_last);
      header(o, whole, piece);
      for (int k = 0; k < np; k++)
        for (int j = 0; j < N1; j++)
          for (int i = 0; i < N0; i++) {
            const long long m = k * N1N0 + (long long)i * N1 + j;
            std::fprintf(o.f, "%.4e %.4e %.4e\n", rx(m), ry(m), rz(m));
          }
      middle(o, nf);
      for (int k = 0; k < np; k++)
        for (int j = 0; j < N1; j++)
          for (int i = 0; i < N0; i++) values_line(o, &vals[(size_t)(k * N1N0 + (long long)i * N1 + j) * nf], nf);
      footer(o);
    }
    std::snprintf(whole, sizeof whole, "<PStructuredGrid WholeExtent=\"0 %d 0 %d 0 %d\" GhostLevel = \"0\" >", N0 - 1, N1 - 1, N2 - 1);
    std::snprintf(piece, sizeof piece, "<Piece Extent=\"0 %d 0 %d %d %d\" Source=\"%%s\" />\n", N0 - 1, N1 - 1, 0, N2 - 1);
    pvts(pv, whole, piece, nf, source);
    return MITHRA_OK;
  }

  double c;
  if (d->plane == 0) {  // plane normal to x, src/fdtd.cpp:1128-1284
    const double fr = std::modf((d->position[0] - d->xmin) / d->dx, &c);
    const int i = (int)c;
    if (i < 0 || i + 1 > N0 - 1) return MITHRA_ERR_ARG;
    std::vector<double> vals((size_t)N1 * np * nf, 0.0);
    for (int k = 0; k < np; k++)
      for (int j = 1; j < N1 - 1; j++) {
        const long long m = k * N1N0 + (long long)i * N1 + j;
        for (int l = 0; l < nf; l++)
          vals[((size_t)k * N1 + j) * nf + l] =
              value(d->field[l], m, en, bn, an, fn) * (1.0 - fr) + value(d->field[l], m + N1, en, bn, an, fn) * fr;
      }
    {
      Out o(vts);
      if (!o.f) return MITHRA_ERR_ARG;
      std::snprintf(whole, sizeof whole, "<StructuredGrid WholeExtent=\"0  0  0 %d %d %d\">", N1 - 1, k0, k_last);
      std::snprintf(piece, sizeof piece, "<Piece Extent=\" 0 0 0 %d %d %d\">", N1 - 1, k0, k_last);
      header(o, whole, piece);
      for (int k = 0; k < np; k++)
        for (int j = 0; j < N1; j++) {
          const long long m = k * N1N0 + (long long)i * N1 + j;
          std::fprintf(o.f, "%.4e %.4e %.4e\n", rx(m) * (1.0 - fr) + rx(m + N1) * fr, ry(m), rz(m));
        }
      middle(o, nf);
      for (int k = 0; k < np; k++)
        for (int j = 0; j < N1; j++) values_line(o, &vals[((size_t)k * N1 + j) * nf], nf);
      footer(o);
    }
    std::snprintf(whole, sizeof whole, "<PStructuredGrid WholeExtent=\" 0 0 0 %d 0 %d\" GhostLevel = \"0\" >", N1 - 1, N2 - 1);
    std::snprintf(piece, sizeof piece, "<Piece Extent=\"0 0 0 %d %d %d\" Source=\"%%s\" />\n", N1 - 1, 0, N2 - 1);
    pvts(pv, whole, piece, nf, source);
    return MITHRA_OK;
  }

  if (d->plane == 1) {  // plane normal to y, src/fdtd.cpp:1290-1446
    const double fr = std::modf((d->position[1] - d->ymin) / d->dy, &c);
    const int j = (int)c;
    if (j < 0 || j + 1 > N1 - 1) return MITHRA_ERR_ARG;
    std::vector<double> vals((size_t)N0 * np * nf, 0.0);
    for (int k = 0; k < np; k++)
      for (int i = 1; i < N0 - 1; i++) {
        const long long m = k * N1N0 + (long long)i * N1 + j;
        for (int l = 0; l < nf; l++)
          vals[((size_t)k * N0 + i) * nf + l] =
              value(d->field[l], m, en, bn, an, fn) * (1.0 - fr) + value(d->field[l], m + 1, en, bn, an, fn) * fr;
      }
    {
      Out o(vts);
      if (!o.f) return MITHRA_ERR_ARG;
      std::snprintf(whole, sizeof whole, "<StructuredGrid WholeExtent=\"0 %d 0 0 %d %d\">", N0 - 1, k0, k_last);
      std::snprintf(piece, sizeof piece, "<Piece Extent=\"0 %d 0 0 %d %d\">", N0 - 1, k0, k_last);
      header(o, whole, piece);
      for (int k = 0; k < np; k++)
        for (int i = 0; i < N0; i++) {
          const long long m = k * N1N0 + (long long)i * N1 + j;
          std::fprintf(o.f, "%.4e %.4e %.4e\n", rx(m) * (1.0 - fr) + rx(m + 1) * fr, ry(m), rz(m));
        }
      middle(o, nf);
      for (int k = 0; k < np; k++)
        for (int i = 0; i < N0; i++) values_line(o, &vals[((size_t)k * N0 + i) * nf], nf);
      footer(o);
    }
    std::snprintf(whole, sizeof whole, "<PStructuredGrid WholeExtent=\"0 %d 0 0 0 %d\" GhostLevel = \"0\" >", N0 - 1, N2 - 1);
    std::snprintf(piece, sizeof piece, "<Piece Extent=\"0 %d 0 0 %d %d\" Source=\"%%s\" />\n", N0 - 1, 0, N2 - 1);
    pvts(pv, whole, piece, nf, source);
    return MITHRA_OK;
  }

  // plane normal to z, src/fdtd.cpp:1452-1540 (no index file)
  const double fr = std::modf((d->position[2] - d->zmin) / d->dz, &c);
  const int k = (int)c - k0;
  if (k < 0 || k + 1 > np - 1) return MITHRA_ERR_ARG;
  std::vector<double> vals((size_t)N1N0 * nf, 0.0);
  for (int j = 1; j < N1 - 1; j++)
    for (int i = 1; i < N0 - 1; i++) {
      const long long m = k * N1N0 + (long long)i * N1 + j;
      for (int l = 0; l < nf; l++)
        vals[((size_t)i * N1 + j) * nf + l] =
            value(d->field[l], m, en, bn, an, fn) * (1.0 - fr) + value(d->field[l], m + N1N0, en, bn, an, fn) * fr;
    }
  Out o(vts);
  if (!o.f) return MITHRA_ERR_ARG;
  std::snprintf(whole, sizeof whole, "<StructuredGrid WholeExtent=\"0 %d 0 %d 0 0\">", N0 - 1, N1 - 1);
  std::snprintf(piece, sizeof piece, "<Piece Extent=\"0 %d 0 %d 0 0\">", N0 - 1, N1 - 1);
  header(o, whole, piece);
  for (int j = 0; j < N1; j++)
    for (int i = 0; i < N0; i++) {
      const long long m = k * N1N0 + (long long)i * N1 + j;
      std::fprintf(o.f, "%.4e %.4e %.4e\n", rx(m) * (1.0 - fr) + rx(m + N1N0) * fr, ry(m), rz(m));
    }
  middle(o, nf);
  for (int j = 0; j < N1; j++)
    for (int i = 0; i < N0; i++) values_line(o, &vals[((size_t)i * N1 + j) * nf], nf);
  footer(o);
  return MITHRA_OK;
}
