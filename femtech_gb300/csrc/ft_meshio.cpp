// ft_meshio.cpp -- mesh input: Abaqus .inp and LS-DYNA .k into the arrays the
// engine takes (host code).
//
// Reference path replaced: ReadInputFile (src/io/input/ReadInputFile.cpp:26-77)
// dispatching on the extension to ReadAbaqus (src/io/input/ReadAbaqus.cpp:26-246)
// or ReadLsDyna (src/io/input/ReadLsDyna.cpp:48-319), followed by the node
// renumbering that PartitionMesh applies on a single rank
// (src/io/PartitionMesh.cpp:485-535, updateConnectivityGlobalToLocal: local
// node j = the j-th smallest node ID used by an element).  The sections,
// tokenisation and column rules follow the reference readers, so a file reads
// into the same arrays; the differences are in cost (one pass over an
// in-memory copy, sort-based renumbering instead of the reference's
// quadratic search) and in what is reported (nodes that no *NODE line
// defines are counted in missing_nodes; the reference leaves them at 0).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <strings.h>
#include <vector>

#include "ftgpu.h"

namespace {

// fgets over an in-memory file with the reference's line buffer
// (MAX_FILE_LINE = 260, include/FemTech.h:19): a longer line comes back in
// pieces of at most 259 characters, as fgets returns it.
constexpr int kMaxLine = 260;
constexpr int kMaxType = 10;     // MAX_ELEMENT_TYPE_SIZE (include/FemTech.h:20)
constexpr int kMaxElset = 80;    // ELSETNAME_SIZE (ReadAbaqus.cpp:103)

struct Reader {
  const char *buf = nullptr;
  size_t size = 0, pos = 0;
  bool gets(std::string &line) {
    if (pos >= size) return false;
    size_t end = pos;
    while (end < size && end - pos < (size_t)kMaxLine - 1) {
      if (buf[end++] == '\n') break;
    }
    line.assign(buf + pos, end - pos);
    pos = end;
    return true;
  }
  long tell() const { return (long)pos; }
  bool seek(long p) {
    if (p < 0 || (size_t)p > size) return false;
    pos = (size_t)p;
    return true;
  }
};

// LineToArray (ReadInputFile.cpp:83-173): numbers of the columns from
// column_to_start (one-based) on; 0 if any token is not a number; with
// check_last, a non-positive value ends the list and a run of more than one
// repeat of the last value is dropped; at most column_count values when > 0.
// Tokens are runs of non-delimiter characters (strtok); each is converted by
// strtod on its own NUL-terminated copy, as the reference converts it.  No
// heap allocation: a line holds at most 259 characters.
int line_to_array(bool check_last, int column_to_start, int column_count,
                  const std::string &line, const char *delim, std::vector<double> *out) {
  double vals[kMaxLine];
  char tok[kMaxLine];
  double last = 2147483647.0;  // INT_MAX
  int column = 0, repeats = 0, result = 0;
  const char *c = line.c_str(), *e = c + line.size();
  while (c < e) {
    while (c < e && strchr(delim, *c)) ++c;
    if (c >= e) break;
    const char *t = c;
    while (c < e && !strchr(delim, *c)) ++c;
    const size_t n = std::min<size_t>(c - t, kMaxLine - 1);
    double v;
    // plain integers (node and element IDs, the bulk of a mesh file) are
    // converted directly: strtod gives the same (exact) value for them
    size_t k = (n > 0 && (t[0] == '-' || t[0] == '+')) ? 1 : 0;
    bool digits = n > k && n - k <= 15;
    long long iv = 0;
    for (size_t q = k; q < n && digits; ++q) {
      if (t[q] < '0' || t[q] > '9') digits = false;
      else iv = iv * 10 + (t[q] - '0');
    }
    if (digits) {
      v = (double)(t[0] == '-' ? -iv : iv);
      if (t[0] == '-' && iv == 0) v = -0.0;
    } else {
      memcpy(tok, t, n);
      tok[n] = 0;
      char *end;
      v = strtod(tok, &end);
      if (end == tok) return 0;
    }
    ++column;
    if (column < column_to_start) continue;
    if (check_last) {
      if (v <= 0) {
        repeats = 0;
        break;
      } else if (v == last) {
        ++repeats;
      } else {
        repeats = 0;
      }
    }
    last = v;
    vals[result++] = v;
  }
  if (result > 0) {
    if (check_last && repeats > 1) result = std::max(0, result - repeats);
    if (column_count > 0 && result > column_count) result = column_count;
  }
  if (out) out->assign(vals, vals + result);
  return result;
}

// LineToTokens (ReadAbaqus.cpp:248-306): words of [A-Za-z0-9_-], every other
// non-blank character a token of its own
void line_tokens(const std::string &line, std::vector<std::string> &tok) {
  tok.clear();
  std::string cur;
  for (char ch : line) {
    if (ch == ' ' || ch == '\t' || ch == '\r' || ch == '\n') {
      if (!cur.empty()) tok.push_back(cur), cur.clear();
    } else if ((ch >= 'a' && ch <= 'z') || (ch >= 'A' && ch <= 'Z') || (ch >= '0' && ch <= '9') ||
               ch == '_' || ch == '-') {
      cur += ch;
    } else {
      if (!cur.empty()) tok.push_back(cur), cur.clear();
      tok.push_back(std::string(1, ch));
    }
  }
  if (!cur.empty()) tok.push_back(cur);
}

// IsLineComplete (ReadAbaqus.cpp:318-328): the last non-blank character is not ','
bool line_complete(const std::string &line) {
  for (int i = (int)line.size() - 1; i >= 0; --i) {
    const char c = line[i];
    if (c == '\r' || c == '\n' || c == ' ' || c == '\t') continue;
    return c != ',';
  }
  return true;
}

// a keyword line's first token is "*" (blanks are not tokens): the test
// that lets every data line skip the tokenisation below
bool starts_with_star(const std::string &line) {
  for (char ch : line) {
    if (ch == ' ' || ch == '\t' || ch == '\r' || ch == '\n') continue;
    return ch == '*';
  }
  return false;
}

// IsNodeSection (ReadAbaqus.cpp:330-347)
bool abq_node_section(std::string &line, Reader &f) {
  if (!starts_with_star(line)) return false;
  std::vector<std::string> t;
  line_tokens(line, t);
  bool r = t.size() >= 2 && t[0] == "*" && strcasecmp(t[1].c_str(), "NODE") == 0;
  if (r && t.size() > 2) {
    r = t[2] == ",";
    if (r)
      while (!line_complete(line) && f.gets(line)) {
      }
  }
  return r;
}

// IsElementSection (ReadAbaqus.cpp:349-378): "*ELEMENT," with TYPE=...
// (ELSET=... optional); continuation lines are read until the header ends.
bool abq_element_section(std::string &line, Reader &f, std::string *type, std::string *elset) {
  if (!starts_with_star(line)) return false;
  std::vector<std::string> t;
  line_tokens(line, t);
  bool r = t.size() > 2 && t[0] == "*" && strcasecmp(t[1].c_str(), "ELEMENT") == 0 && t[2] == ",";
  if (!r) return false;
  r = false;
  while (true) {
    for (size_t i = 0; i < t.size(); ++i) {
      if (!r && strcasecmp(t[i].c_str(), "TYPE") == 0) {
        r = i + 2 < t.size() && t[i + 1] == "=" && !t[i + 2].empty();
        if (r && type) *type = t[i + 2];
      }
      if (strcasecmp(t[i].c_str(), "ELSET") == 0 && i + 2 < t.size() && t[i + 1] == "=" && elset)
        *elset = t[i + 2];
    }
    if (line_complete(line)) break;
    if (!f.gets(line)) break;  // (the reference loops on the last line at end of file)
    if (!r) line_tokens(line, t);
  }
  return r;
}

int type_code(const std::string &t) {
  if (t == "C3D8") return FTGPU_C3D8;
  if (t == "C3D4") return FTGPU_C3D4;
  if (t == "T3D2") return FTGPU_T3D2;
  return -1;
}

// Raw reader output: per element its node IDs (0-based, as in the file minus
// one), part, type and ID; coordinates of the used node IDs.
struct Raw {
  int ndim = 0;
  std::vector<int> eptr{0}, conn, pid, etype, eid;
  std::vector<int> uniq;          // sorted unique node IDs used by elements
  std::vector<double> ucoord;     // ndim per unique ID
  long long missing = 0;
};

// sorted unique IDs of the connectivity, for the node pass
void unique_ids(Raw &r) {
  r.uniq = r.conn;
  std::sort(r.uniq.begin(), r.uniq.end());
  r.uniq.erase(std::unique(r.uniq.begin(), r.uniq.end()), r.uniq.end());
  r.ucoord.assign(r.uniq.size() * (size_t)r.ndim, 0.0);
}

int idx_of(const std::vector<int> &u, int id) {
  auto it = std::lower_bound(u.begin(), u.end(), id);
  return (it != u.end() && *it == id) ? (int)(it - u.begin()) : -1;
}

// ReadAbaqus, one rank (ReadAbaqus.cpp:26-246)
bool read_abaqus(Reader &f, Raw &r, std::string &err) {
  const char *delim = ", \t";
  std::string line;
  long elem_pos = -1, node_pos = -1, cur = f.tell();
  int nall = 0;
  std::vector<double> v;
  while (f.gets(line)) {
    if (node_pos == -1 && abq_node_section(line, f)) {
      const long p = f.tell();
      if (f.gets(line)) {
        const int n = line_to_array(false, 1, 0, line, delim, nullptr) - 1;
        if (n >= 2) {
          r.ndim = n > 3 ? 3 : n;
          node_pos = p;
        }
      }
    }
    if (abq_element_section(line, f, nullptr, nullptr)) {
      if (elem_pos == -1) elem_pos = cur;
      long last = -1;
      while (f.gets(line)) {
        if (line_to_array(false, 2, 0, line, delim, nullptr) == 0) break;
        ++nall;
        last = f.tell();
      }
      f.seek(last);
    }
    if (elem_pos == -1) cur = f.tell();
  }
  if (nall == 0) err = "no element found";
  else if (node_pos == -1) err = "node section not found";
  if (nall == 0 || node_pos == -1 || !f.seek(elem_pos)) return false;
  // elements: node IDs, element set -> part (order of first appearance), type
  std::string type, elset;
  std::vector<std::string> sets;
  while (f.gets(line)) {
    if (!abq_element_section(line, f, &type, &elset)) continue;
    // the reference matches the name against every slot of its name table,
    // unfilled (empty) slots included: an empty name (a section without
    // ELSET before any named one, or an ELSET given only on a continuation
    // line) is never added and its elements keep part 0
    std::string name = elset.substr(0, kMaxElset - 1);
    int part = name.empty() ? 0 : -1;
    for (size_t k = 0; k < sets.size() && part < 0; ++k)
      if (sets[k] == name) part = (int)k;
    if (part < 0) {
      sets.push_back(name);
      part = (int)sets.size() - 1;
    }
    const int code = type_code(type.substr(0, kMaxType - 1));
    long last = -1;
    while (f.gets(line)) {
      const int n = line_to_array(false, 1, 0, line, delim, &v);
      if (line_to_array(false, 2, 0, line, delim, nullptr) == 0 || n < 2) break;
      r.eid.push_back((int)v[0]);
      for (int k = 1; k < n; ++k) r.conn.push_back((int)v[k] - 1);
      r.eptr.push_back((int)r.conn.size());
      r.pid.push_back(part);
      r.etype.push_back(code);
      last = f.tell();
    }
    f.seek(last);
  }
  // nodes: the first *NODE section, lines of exactly ndim + 1 numbers
  unique_ids(r);
  f.seek(node_pos);
  const int ncols = r.ndim + 1;
  size_t copied = 0;
  std::vector<char> seen(r.uniq.size(), 0);
  while (copied < r.uniq.size() && f.gets(line)) {
    const int n = line_to_array(false, 1, ncols, line, delim, &v);
    if (n != ncols) break;
    const int I = idx_of(r.uniq, (int)v[0] - 1);
    if (I >= 0) {
      for (int d = 0; d < r.ndim; ++d) r.ucoord[(size_t)I * r.ndim + d] = v[1 + d];
      seen[I] = 1;
      ++copied;
    }
  }
  for (char s : seen) r.missing += s ? 0 : 1;
  return true;
}

// ReadLsDyna, one rank (ReadLsDyna.cpp:48-319)
bool dyna_element_section(std::string &line, Reader &f, int *beam) {
  static const char *kTitles[3] = {"*ELEMENT_SOLID", "*ELEMENT_SHELL", "*ELEMENT_BEAM"};
  bool r = false;
  for (const char *t : kTitles) r = r || line.compare(0, strlen(t), t) == 0;
  if (r) {
    if (beam && line.compare(0, strlen(kTitles[2]), kTitles[2]) == 0) *beam = 1;
    f.gets(line);  // the line after the keyword (the column comment) is skipped
  }
  return r;
}

int distinct(const std::vector<double> &a) {  // CalcUniqueValues (ReadLsDyna.cpp:34-46)
  int r = 1;
  for (size_t i = 1; i < a.size(); ++i) {
    size_t j = 0;
    for (; j < i; ++j)
      if (a[i] == a[j]) break;
    if (i == j) ++r;
  }
  return r;
}

bool read_lsdyna(Reader &f, Raw &r, std::string &err) {
  const char *delim = " \t";
  std::string line;
  long elem_pos = -1, node_pos = -1, cur = f.tell();
  int beam = 0, nall = 0;
  std::vector<double> v;
  r.ndim = 0;
  while (f.gets(line)) {
    if (dyna_element_section(line, f, &beam)) {
      if (elem_pos == -1) elem_pos = cur;
      long last = -1;
      while (f.gets(line)) {
        if (line_to_array(false, 2, 1, line, delim, nullptr) == 0 ||
            line_to_array(true, 3, 0, line, delim, nullptr) == 0)
          break;
        ++nall;
        last = f.tell();
      }
      f.seek(last);
    } else if (node_pos == -1 && line.compare(0, 5, "*NODE") == 0) {
      bool dim3 = false;
      while (!dim3 && f.gets(line)) {
        if (r.ndim == 0 && line.find("nid") != std::string::npos) {
          if (line.find('x') != std::string::npos) ++r.ndim;
          if (line.find('y') != std::string::npos) ++r.ndim;
          if (line.find('z') != std::string::npos) ++r.ndim;
          if (r.ndim == 2 || r.ndim == 3) node_pos = f.tell();
        } else if (r.ndim == 3) {
          if (line_to_array(false, 4, 1, line, delim, &v) > 0) dim3 = v[0] != 0;
        }
      }
      if ((r.ndim == 2 || r.ndim == 3) && !dim3 && beam == 0) r.ndim = 2;
    }
    if (elem_pos == -1) cur = f.tell();
  }
  if (nall == 0) err = "no element found";
  else if (node_pos == -1) err = "node section not found";
  if (nall == 0 || node_pos == -1 || !f.seek(elem_pos)) return false;
  std::vector<double> nodes;
  while (f.gets(line)) {
    if (!dyna_element_section(line, f, nullptr)) continue;
    long last = -1;
    while (f.gets(line)) {
      const int ne = line_to_array(false, 1, 1, line, delim, &v);
      const double eid = ne > 0 ? v[0] : 0.0;
      const int np = line_to_array(false, 2, 1, line, delim, &v);
      const double part = np > 0 ? v[0] : 0.0;
      const int nn = line_to_array(true, 3, 0, line, delim, &nodes);
      if (np == 0 || nn == 0 || ne == 0) break;
      r.eid.push_back((int)eid);
      r.pid.push_back((int)part - 1);
      const int N = nn == 8 ? distinct(nodes) : nn;
      r.etype.push_back(N > 4 ? FTGPU_C3D8 : (N == 4 ? FTGPU_C3D4 : (N == 2 ? FTGPU_T3D2 : -1)));
      for (int k = 0; k < nn; ++k) r.conn.push_back((int)nodes[k] - 1);
      r.eptr.push_back((int)r.conn.size());
      last = f.tell();
    }
    f.seek(last);
  }
  unique_ids(r);
  f.seek(node_pos);
  const int ncols = r.ndim + 1;
  size_t copied = 0;
  std::vector<char> seen(r.uniq.size(), 0);
  while (copied < r.uniq.size() && f.gets(line)) {
    const int n = line_to_array(false, 1, ncols, line, delim, &v);
    if (n == ncols) {
      const int I = idx_of(r.uniq, (int)v[0] - 1);
      if (I >= 0) {
        for (int d = 0; d < r.ndim; ++d) r.ucoord[(size_t)I * r.ndim + d] = v[1 + d];
        seen[I] = 1;
        ++copied;
      }
    }
    if (line.compare(0, 4, "*END") == 0) break;
  }
  for (char s : seen) r.missing += s ? 0 : 1;
  return true;
}

thread_local std::string g_err;

template <class T>
T *copy_out(const std::vector<T> &v) {
  T *p = (T *)malloc(std::max<size_t>(1, v.size()) * sizeof(T));
  if (p && !v.empty()) memcpy(p, v.data(), v.size() * sizeof(T));
  return p;
}

}  // namespace

extern "C" {

int ftgpu_read_mesh(const char *path, ftgpu_mesh **out) {
  if (!path || !out) return FTGPU_ERR_INPUT;
  *out = nullptr;
  const char *dot = strrchr(path, '.');
  const char *ext = dot ? dot : "";
  const bool dyna = strcasecmp(ext, ".k") == 0, abq = strcasecmp(ext, ".inp") == 0;
  if (!dyna && !abq) {
    g_err = "input file type is unknown (.inp or .k)";
    return FTGPU_ERR_INPUT;
  }
  FILE *fp = fopen(path, "rb");
  if (!fp) {
    g_err = std::string("cannot open ") + path;
    return FTGPU_ERR_INPUT;
  }
  std::vector<char> data;
  char chunk[1 << 16];
  size_t got;
  while ((got = fread(chunk, 1, sizeof(chunk), fp)) > 0) data.insert(data.end(), chunk, chunk + got);
  fclose(fp);
  Reader f;
  f.buf = data.data();
  f.size = data.size();
  Raw r;
  std::string err;
  const bool ok = dyna ? read_lsdyna(f, r, err) : read_abaqus(f, r, err);
  if (!ok) {
    g_err = "mesh read failed: " + err;
    return FTGPU_ERR_INPUT;
  }
  // single-rank PartitionMesh: local node j = j-th smallest used node ID
  ftgpu_mesh *m = (ftgpu_mesh *)calloc(1, sizeof(ftgpu_mesh));
  if (!m) return FTGPU_ERR_ALLOC;
  m->ndim = r.ndim;
  m->nNodes = (int)r.uniq.size();
  m->nelements = (int)r.pid.size();
  std::vector<int> local(r.conn.size());
  for (size_t k = 0; k < r.conn.size(); ++k) local[k] = idx_of(r.uniq, r.conn[k]);
  std::vector<int> gid(r.uniq.size());
  for (size_t k = 0; k < r.uniq.size(); ++k) gid[k] = r.uniq[k] + 1;
  std::vector<int> parts = r.pid;
  std::sort(parts.begin(), parts.end());
  parts.erase(std::unique(parts.begin(), parts.end()), parts.end());
  m->nPID = (int)parts.size();                                // ReadInputFile.cpp:59-64
  m->nPIDglobal = parts.empty() ? 0 : parts.back() + 1;
  m->missing_nodes = r.missing;
  m->coordinates = copy_out(r.ucoord);
  m->eptr = copy_out(r.eptr);
  m->connectivity = copy_out(local);
  m->etype = copy_out(r.etype);
  m->pid = copy_out(r.pid);
  m->global_eid = copy_out(r.eid);
  m->global_node_id = copy_out(gid);
  if (!m->coordinates || !m->eptr || !m->connectivity || !m->etype || !m->pid ||
      !m->global_eid || !m->global_node_id) {
    ftgpu_free_mesh(m);
    return FTGPU_ERR_ALLOC;
  }
  *out = m;
  return FTGPU_OK;
}

void ftgpu_free_mesh(ftgpu_mesh *m) {
  if (!m) return;
  free(m->coordinates);
  free(m->eptr);
  free(m->connectivity);
  free(m->etype);
  free(m->pid);
  free(m->global_eid);
  free(m->global_node_id);
  free(m);
}

const char *ftgpu_read_mesh_error(void) { return g_err.c_str(); }

}  // extern "C"
