// ft_vtu.cpp -- output steps: the reference's ASCII VTU / PVTU / PVD files
// (host code).
//
// Reference path replaced: WriteVTU (src/io/output/WriteVTU.cpp:3-263) and
// WritePVD (src/io/output/WritePVD.cpp:6-36) on one rank: the same files,
// names and text (the printf formats are kept, so the bytes match), written
// from arrays.  The text of the large arrays is formatted by several host
// threads into per-range buffers and written in order.
#include <sys/stat.h>

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "ftgpu.h"

namespace {

// rows [0, n) formatted by fmt_row into one string, split over threads
template <class F>
std::string format_rows(long long n, F fmt_row) {
  const int nt = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  const long long per = (n + nt - 1) / nt;
  std::vector<std::string> part(nt);
  std::vector<std::thread> th;
  for (int t = 0; t < nt; ++t)
    th.emplace_back([&, t] {
      const long long b = t * per, e = std::min(n, b + per);
      std::string &s = part[t];
      char line[1024];
      for (long long i = b; i < e; ++i) {
        const int k = fmt_row(i, line, sizeof(line));
        s.append(line, std::min<size_t>(k > 0 ? (size_t)k : 0, sizeof(line) - 1));
      }
    });
  for (auto &x : th) x.join();
  std::string out;
  size_t total = 0;
  for (auto &p : part) total += p.size();
  out.reserve(total);
  for (auto &p : part) out += p;
  return out;
}

int mkdirs(const std::string &path) {
  std::string cur;
  for (size_t i = 0; i <= path.size(); ++i) {
    if (i == path.size() || path[i] == '/') {
      if (!cur.empty() && mkdir(cur.c_str(), 0755) != 0 && errno != EEXIST) return -1;
    }
    if (i < path.size()) cur += path[i];
  }
  return 0;
}

int vtk_type(int etype) { return etype == FTGPU_C3D8 ? 12 : (etype == FTGPU_C3D4 ? 10 : 3); }

}  // namespace

extern "C" {

int ftgpu_write_vtu_arrays(const char *dir, const char *name, int step, int nNodes,
                           int nelements, const double *coordinates, const int *eptr,
                           const int *connectivity, const int *etype, const int *pid,
                           const double *u, const double *a, const int *boundary,
                           const double *Eavg, int ncell, const int *const *cell_data,
                           const char *const *cell_names) {
  if (!name || nNodes <= 0 || nelements <= 0 || !coordinates || !eptr || !connectivity ||
      !etype || !pid || !u || !a || !boundary || !Eavg || (ncell > 0 && (!cell_data || !cell_names)))
    return FTGPU_ERR_INPUT;
  const std::string root = dir && *dir ? std::string(dir) + "/" : std::string("./");
  if (mkdirs(root + "results/vtu")) return FTGPU_ERR_INPUT;
  char s[64];
  snprintf(s, sizeof(s), ".vtu.%04d.%04d", step, 0);
  const std::string vtu = root + "results/vtu/" + name + s;
  FILE *fp = fopen(vtu.c_str(), "w");
  if (!fp) return FTGPU_ERR_INPUT;
  const int nd = 3;
  fprintf(fp, "<?xml version=\"1.0\"?>\n");
  fprintf(fp, "<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\">\n");
  fprintf(fp, "\t<UnstructuredGrid>\n");
  fprintf(fp, "\t\t<Piece NumberOfPoints=\"%d\" NumberOfCells=\"%d\">\n", nNodes, nelements);
  fprintf(fp, "\t\t\t<Points>\n");
  fprintf(fp, "\t\t\t\t<DataArray type=\"Float64\" NumberOfComponents=\"%d\" format=\"ascii\">\n", nd);
  // deformed positions; displacements below 1e-20 in magnitude are written as
  // 0 (the reference flushes them in its displacement array while writing)
  auto flushed = [&](long long k) { return std::fabs(u[k] - 0.0) < 1e-20 ? 0.0 : u[k]; };
  std::string t = format_rows(nNodes, [&](long long i, char *b, size_t n) {
    return snprintf(b, n, "\t\t\t\t\t%10.8e %10.8e %10.8e \n", coordinates[3 * i] + flushed(3 * i),
                    coordinates[3 * i + 1] + flushed(3 * i + 1),
                    coordinates[3 * i + 2] + flushed(3 * i + 2));
  });
  fwrite(t.data(), 1, t.size(), fp);
  fprintf(fp, "\t\t\t\t</DataArray>\n");
  fprintf(fp, "\t\t\t</Points>\n");
  fprintf(fp, "\t\t\t<Cells>\n");
  fprintf(fp, "\t\t\t\t<DataArray type=\"Int32\" Name=\"connectivity\" format=\"ascii\">\n");
  t = format_rows(nelements, [&](long long e, char *b, size_t n) {
    int k = snprintf(b, n, "\t\t\t\t\t");
    for (int j = eptr[e]; j < eptr[e + 1] && k < (int)n - 16; ++j)
      k += snprintf(b + k, n - k, "%d ", connectivity[j]);
    k += snprintf(b + k, n - k, "\n");
    return k;
  });
  fwrite(t.data(), 1, t.size(), fp);
  fprintf(fp, "\t\t\t\t</DataArray>\n");
  fprintf(fp, "\t\t\t\t<DataArray type=\"Int32\" Name=\"offsets\" format=\"ascii\">\n");
  t = format_rows(nelements, [&](long long e, char *b, size_t n) {
    return snprintf(b, n, "\t\t\t\t\t%d\n", eptr[e + 1]);
  });
  fwrite(t.data(), 1, t.size(), fp);
  fprintf(fp, "\t\t\t\t</DataArray>\n");
  fprintf(fp, "\t\t\t\t<DataArray type=\"Int32\" Name=\"types\" format=\"ascii\">\n");
  t = format_rows(nelements, [&](long long e, char *b, size_t n) {
    return snprintf(b, n, "\t\t\t\t\t%d\n", vtk_type(etype[e]));
  });
  fwrite(t.data(), 1, t.size(), fp);
  fprintf(fp, "\t\t\t\t</DataArray>\n");
  fprintf(fp, "\t\t\t</Cells>\n");
  fprintf(fp, "\t\t\t<PointData>\n");
  const char *vec_hdr =
      "\t\t\t\t<DataArray type=\"%s\" Name=\"%s\" NumberOfComponents=\"%d\" ComponentName0=\"X\" "
      "ComponentName1=\"Y\" ComponentName2=\"Z\" format=\"ascii\">\n";
  fprintf(fp, vec_hdr, "Float64", "Displacements", nd);
  t = format_rows(nNodes, [&](long long i, char *b, size_t n) {
    return snprintf(b, n, "\t\t\t\t\t%10.8e %10.8e %10.8e \n", flushed(3 * i), flushed(3 * i + 1),
                    flushed(3 * i + 2));
  });
  fwrite(t.data(), 1, t.size(), fp);
  fprintf(fp, "\t\t\t\t</DataArray>\n");
  fprintf(fp, vec_hdr, "Float64", "Accelerations", nd);
  t = format_rows(nNodes, [&](long long i, char *b, size_t n) {
    return snprintf(b, n, "\t\t\t\t\t%10.8e %10.8e %10.8e \n", a[3 * i], a[3 * i + 1], a[3 * i + 2]);
  });
  fwrite(t.data(), 1, t.size(), fp);
  fprintf(fp, "\t\t\t\t</DataArray>\n");
  fprintf(fp, vec_hdr, "Int32", "Boundary", nd);
  t = format_rows(nNodes, [&](long long i, char *b, size_t n) {
    return snprintf(b, n, "\t\t\t\t\t%d %d %d \n", boundary[3 * i], boundary[3 * i + 1],
                    boundary[3 * i + 2]);
  });
  fwrite(t.data(), 1, t.size(), fp);
  fprintf(fp, "\t\t\t\t</DataArray>\n");
  fprintf(fp, "\t\t\t</PointData>\n");
  fprintf(fp, "\t\t\t<CellData>\n");
  fprintf(fp, "\t\t\t\t<DataArray type=\"Int32\" Name=\"PartID\" format=\"ascii\">\n");
  t = format_rows(nelements, [&](long long e, char *b, size_t n) {
    return snprintf(b, n, "\t\t\t\t\t%d\n", pid[e]);
  });
  fwrite(t.data(), 1, t.size(), fp);
  fprintf(fp, "\t\t\t\t</DataArray>\n");
  fprintf(fp,
          "\t\t\t\t<DataArray type=\"Float64\" Name=\"AvgStrain\" NumberOfComponents=\"%d\" "
          "ComponentName0=\"E11\" ComponentName1=\"E21\" ComponentName2=\"E31\" "
          "ComponentName3=\"E12\" ComponentName4=\"E22\" ComponentName5=\"E32\" "
          "ComponentName6=\"E13\" ComponentName7=\"E23\" ComponentName8=\"E33\" "
          "format=\"ascii\">\n",
          nd * nd);
  t = format_rows(nelements, [&](long long e, char *b, size_t n) {
    const double *E = Eavg + 9 * e;
    return snprintf(b, n,
                    "\t\t\t\t\t%10.8e %10.8e %10.8e %10.8e %10.8e %10.8e %10.8e %10.8e %10.8e \n",
                    E[0], E[1], E[2], E[3], E[4], E[5], E[6], E[7], E[8]);
  });
  fwrite(t.data(), 1, t.size(), fp);
  fprintf(fp, "\t\t\t\t</DataArray>\n");
  fprintf(fp, "\t\t\t\t<DataArray type=\"Int32\" Name=\"ProcID\" format=\"ascii\">\n");
  t = format_rows(nelements, [&](long long, char *b, size_t n) {
    return snprintf(b, n, "\t\t\t\t\t%d\n", 0);
  });
  fwrite(t.data(), 1, t.size(), fp);
  fprintf(fp, "\t\t\t\t</DataArray>\n");
  for (int c = 0; c < ncell; ++c) {
    const int *d = cell_data[c];
    fprintf(fp, "\t\t\t\t<DataArray type=\"Int32\" Name=\"%s\" format=\"ascii\">\n", cell_names[c]);
    t = format_rows(nelements, [&](long long e, char *b, size_t n) {
      return snprintf(b, n, "\t\t\t\t\t%d\n", d[e]);
    });
    fwrite(t.data(), 1, t.size(), fp);
    fprintf(fp, "\t\t\t\t</DataArray>\n");
  }
  fprintf(fp, "\t\t\t</CellData>\n");
  fprintf(fp, "\t\t</Piece>\n");
  fprintf(fp, "\t</UnstructuredGrid>\n");
  fprintf(fp, "</VTKFile>\n");
  const bool werr = ferror(fp) != 0;
  fclose(fp);
  if (werr) return FTGPU_ERR_INPUT;

  // the parallel collection file (rank 0), one piece
  snprintf(s, sizeof(s), ".%.04d.pvtu", step);
  fp = fopen((root + "results/" + name + s).c_str(), "w");
  if (!fp) return FTGPU_ERR_INPUT;
  fprintf(fp, "<?xml version=\"1.0\"?>\n");
  fprintf(fp, "<VTKFile type=\"PUnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\">\n");
  fprintf(fp, "\t<PUnstructuredGrid GhostLevel=\"0\">\n");
  fprintf(fp, "\t\t<PPoints>\n");
  fprintf(fp, "\t\t\t<PDataArray type=\"Float64\" NumberOfComponents=\"%d\" format=\"ascii\"/>\n", nd);
  fprintf(fp, "\t\t</PPoints>\n");
  fprintf(fp, "\t\t<PCells>\n");
  fprintf(fp, "\t\t\t<PDataArray type=\"Int32\" Name=\"connectivity\" NumberOfComponents=\"1\"/>\n");
  fprintf(fp, "\t\t\t<PDataArray type=\"Int32\" Name=\"offsets\" NumberOfComponents=\"1\"/>\n");
  fprintf(fp, "\t\t\t<PDataArray type=\"Int32\" Name=\"types\" NumberOfComponents=\"1\"/>\n");
  fprintf(fp, "\t\t</PCells>\n");
  fprintf(fp, "\t\t<PPointData  Vectors=\"Displacements Accelerations\" >\n");
  const char *pvec =
      "\t\t\t<PDataArray type=\"%s\" Name=\"%s\" NumberOfComponents=\"%d\" ComponentName0=\"X\" "
      "ComponentName1=\"Y\" ComponentName2=\"Z\" format=\"ascii\" />\n";
  fprintf(fp, pvec, "Float64", "Displacements", nd);
  fprintf(fp, pvec, "Float64", "Accelerations", nd);
  fprintf(fp, pvec, "Int32", "Boundary", nd);
  fprintf(fp, "\t\t</PPointData>\n");
  fprintf(fp, "\t\t<PCellData Scalars=\"PartID\" Tensors=\"AvgStrain\">\n");
  fprintf(fp, "\t\t\t<PDataArray type=\"Int32\" Name=\"PartID\"/>\n");
  fprintf(fp,
          "\t\t\t<PDataArray type=\"Float64\" Name=\"AvgStrain\" NumberOfComponents=\"%d\" "
          "ComponentName0=\"E11\" ComponentName1=\"E21\" ComponentName2=\"E31\" "
          "ComponentName3=\"E12\" ComponentName4=\"E22\" ComponentName5=\"E32\" "
          "ComponentName6=\"E13\" ComponentName7=\"E23\" ComponentName8=\"E33\" "
          "format=\"ascii\"/>\n",
          nd * nd);
  fprintf(fp, "\t\t\t<PDataArray type=\"Int32\" Name=\"ProcID\"/>\n");
  for (int c = 0; c < ncell; ++c)
    fprintf(fp, "\t\t\t<PDataArray type=\"Int32\" Name=\"%s\"/>\n", cell_names[c]);
  fprintf(fp, "\t\t</PCellData>\n");
  fprintf(fp, "\t\t<Piece Source=\"vtu/%s.vtu.%04d.%.4d\"/>\n", name, step, 0);
  fprintf(fp, "\t</PUnstructuredGrid>\n");
  fprintf(fp, "</VTKFile>\n");
  fclose(fp);
  return FTGPU_OK;
}

int ftgpu_write_pvd(const char *dir, const char *name, int step, const double *step_time) {
  if (!name || step < 0 || !step_time) return FTGPU_ERR_INPUT;
  std::string base(name);  // strip_ext (WritePVD.cpp:38-46)
  for (size_t i = base.size(); i > 0; --i) {
    const char c = base[i - 1];
    if (c == '\\' || c == '/') break;
    if (c == '.') {
      if (i - 1 > 0) base.resize(i - 1);
      break;
    }
  }
  const std::string root = dir && *dir ? std::string(dir) + "/" : std::string("./");
  FILE *fp = fopen((root + base + ".pvd").c_str(), "w");
  if (!fp) return FTGPU_ERR_INPUT;
  fprintf(fp, "<?xml version=\"1.0\"?>\n");
  fprintf(fp, "<VTKFile type=\"Collection\" version=\"0.1\" "
              "byte_order=\"LittleEndian\" compressor=\"vtkZLibDataCompressor\" >\n");
  fprintf(fp, "\t<Collection>\n");
  for (int j = 0; j < step + 1; ++j)
    fprintf(fp, "\t\t<DataSet timestep=\"%f\" file=\"results/%s.%.04d.pvtu\" />\n", step_time[j],
            base.c_str(), j);
  fprintf(fp, "\t</Collection>\n");
  fprintf(fp, "</VTKFile>\n");
  fclose(fp);
  return FTGPU_OK;
}

}  // extern "C"
