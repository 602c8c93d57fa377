// ckpt.cpp -- the resident state in the reference's checkpoint variable file
// format (variables.bin, written by checkpoint_write_vl,
// src/main/checkpoint/checkpoint_save.c:412-470, and read by
// checkpoint_load_Vars, src/main/checkpoint/checkpoint_load.c:397-500), so
// that GPU runs can restart from the reference's checkpoints and the
// reference can restart from theirs.
//
// Format: a text header ("number of variables and variable list in this
// file:", the count, one variable name per line, a blank line pair,
// "variable-list-data:", a blank line), then per element "{", the element
// name, the number of points, and per variable its index in the list
// ("i", or "i n0 n1 n2" for arrays of other sizes) followed by the raw
// little-endian doubles and a newline, then "}" and a blank line; finally
// "EndOfFile.".  The scalar wave's variables are written in the reference's
// variable-database order (phi, pi, cx, cy, cz).
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/nmg.h"
#include "mesh.h"

namespace {

const char *kVarNames[NMG_NFIELDS] = {"scalarwave1_phi", "scalarwave1_pi", "scalarwave1_cx",
                                      "scalarwave1_cy", "scalarwave1_cz"};
const int kVarField[NMG_NFIELDS] = {4, 0, 1, 2, 3};  // file variable -> state field

std::string g_ckpt_err;
int fail(int code, const std::string &msg) {
  g_ckpt_err = msg;
  return code;
}

bool little_endian() {
  const uint16_t x = 1;
  unsigned char b;
  std::memcpy(&b, &x, 1);
  return b == 1;
}

void to_le(const double *src, size_t n, std::vector<unsigned char> *out) {
  out->resize(n * 8);
  std::memcpy(out->data(), src, n * 8);
  if (!little_endian())
    for (size_t i = 0; i < n; i++)
      for (int k = 0; k < 4; k++) std::swap((*out)[i * 8 + k], (*out)[i * 8 + 7 - k]);
}

void from_le(const unsigned char *src, size_t n, double *dst) {
  std::memcpy(dst, src, n * 8);
  if (!little_endian()) {
    unsigned char *b = reinterpret_cast<unsigned char *>(dst);
    for (size_t i = 0; i < n; i++)
      for (int k = 0; k < 4; k++) std::swap(b[i * 8 + k], b[i * 8 + 7 - k]);
  }
}

std::string elem_name(const nmg_mesh *m, const char *const *names, int64_t e) {
  if (names) return names[e];
  return m->names.empty() ? std::string() : m->names[e];
}

// one text line (without the newline) starting at *pos
bool get_line(const std::vector<unsigned char> &b, size_t *pos, std::string *line) {
  if (*pos >= b.size()) return false;
  size_t q = *pos;
  while (q < b.size() && b[q] != '\n') q++;
  line->assign(reinterpret_cast<const char *>(b.data()) + *pos, q - *pos);
  *pos = q < b.size() ? q + 1 : q;
  return true;
}

}  // namespace

extern "C" {

const char *nmg_checkpoint_last_error(void) { return g_ckpt_err.c_str(); }

const char *nmg_mesh_element_name(const nmg_mesh *m, int64_t e) {
  if (!m || e < 0 || e >= m->nelem || m->names.empty()) return nullptr;
  return m->names[e].c_str();
}

int nmg_checkpoint_write_host(const nmg_mesh *m, const double *u, const char *path,
                              const char *const *names) {
  if (!m || !u || !path) return fail(NMG_EINVAL, "nmg_checkpoint_write_host: null argument");
  if (!names && m->names.empty())
    return fail(NMG_EINVAL, "nmg_checkpoint_write_host: the mesh has no element names");
  FILE *fp = std::fopen(path, "wb");
  if (!fp) return fail(NMG_EINVAL, std::string("cannot open ") + path);
  const int np = m->n * m->n * m->n;
  std::fprintf(fp, "number of variables and variable list in this file:\n");
  std::fprintf(fp, "%d\n", NMG_NFIELDS);
  for (int v = 0; v < NMG_NFIELDS; v++) std::fprintf(fp, "%s\n", kVarNames[v]);
  std::fprintf(fp, "\n\n");
  std::fprintf(fp, "variable-list-data:\n\n");
  std::vector<unsigned char> le;
  for (int64_t e = 0; e < m->nelem; e++) {
    std::fprintf(fp, "{\n%s\n%d\n", elem_name(m, names, e).c_str(), np);
    for (int v = 0; v < NMG_NFIELDS; v++) {
      std::fprintf(fp, "%d\n", v);
      to_le(u + ((size_t)e * NMG_NFIELDS + kVarField[v]) * np, np, &le);
      std::fwrite(le.data(), 1, le.size(), fp);
      std::fprintf(fp, "\n");
    }
    std::fprintf(fp, "}\n\n");
  }
  std::fprintf(fp, "EndOfFile.\n");
  if (std::fclose(fp) != 0) return fail(NMG_EINVAL, std::string("write error on ") + path);
  return NMG_OK;
}

int nmg_checkpoint_read_host(const nmg_mesh *m, const char *path, double *u,
                             const char *const *names) {
  if (!m || !u || !path) return fail(NMG_EINVAL, "nmg_checkpoint_read_host: null argument");
  if (!names && m->names.empty())
    return fail(NMG_EINVAL, "nmg_checkpoint_read_host: the mesh has no element names");
  FILE *fp = std::fopen(path, "rb");
  if (!fp) return fail(NMG_EINVAL, std::string("cannot open ") + path);
  std::vector<unsigned char> b;
  {
    unsigned char buf[1 << 16];
    size_t k;
    while ((k = std::fread(buf, 1, sizeof buf, fp)) > 0) b.insert(b.end(), buf, buf + k);
    std::fclose(fp);
  }
  const int np = m->n * m->n * m->n;
  size_t pos = 0;
  std::string line;
  if (!get_line(b, &pos, &line) || line.rfind("number of variables", 0) != 0)
    return fail(NMG_EINVAL, "not a variable checkpoint file (header)");
  if (!get_line(b, &pos, &line)) return fail(NMG_EINVAL, "truncated header");
  const int nv = std::atoi(line.c_str());
  std::vector<int> field(nv > 0 ? nv : 0, -1);  // file variable -> state field
  for (int v = 0; v < nv; v++) {
    if (!get_line(b, &pos, &line)) return fail(NMG_EINVAL, "truncated variable list");
    for (int k = 0; k < NMG_NFIELDS; k++)
      if (line == kVarNames[k]) field[v] = kVarField[k];
  }
  for (int k = 0; k < NMG_NFIELDS; k++) {
    bool found = false;
    for (int v = 0; v < nv; v++) found = found || field[v] == kVarField[k];
    if (!found) return fail(NMG_EINVAL, std::string("variable ") + kVarNames[k] + " missing");
  }
  while (get_line(b, &pos, &line) && line != "variable-list-data:") {}
  std::unordered_map<std::string, int64_t> index;
  for (int64_t e = 0; e < m->nelem; e++) index[elem_name(m, names, e)] = e;
  std::vector<char> seen(m->nelem, 0);
  int64_t nseen = 0;
  while (get_line(b, &pos, &line)) {
    if (line.empty()) continue;
    if (line == "EndOfFile.") break;
    if (line != "{") return fail(NMG_EINVAL, "malformed element block");
    if (!get_line(b, &pos, &line)) return fail(NMG_EINVAL, "truncated element block");
    auto it = index.find(line);
    if (it == index.end()) return fail(NMG_EMESH, "element " + line + " is not in the mesh");
    const int64_t e = it->second;
    if (!get_line(b, &pos, &line) || std::atoi(line.c_str()) != np)
      return fail(NMG_EMESH, "element points differ from the mesh's n^3");
    while (get_line(b, &pos, &line) && line != "}") {
      int vli = -1, n0 = 0, n1 = 0, n2 = 0;
      const int got = std::sscanf(line.c_str(), "%d %d %d %d", &vli, &n0, &n1, &n2);
      if (got < 1 || vli < 0 || vli >= nv) return fail(NMG_EINVAL, "bad variable index");
      if (got == 4 && (n0 <= 0 || n1 <= 0 || n2 <= 0))
        return fail(NMG_EINVAL, "bad variable dimensions");
      // the doubles left in the file bound every partial product, so the
      // element count is formed without overflow
      const size_t avail = pos <= b.size() ? (b.size() - pos) / 8 : 0;
      size_t cnt = (size_t)np;
      if (got == 4) {
        if ((size_t)n0 > avail || (size_t)n1 > avail / (size_t)n0 ||
            (size_t)n2 > avail / ((size_t)n0 * (size_t)n1))
          return fail(NMG_EINVAL, "truncated variable data");
        cnt = (size_t)n0 * (size_t)n1 * (size_t)n2;
      }
      if (cnt > avail) return fail(NMG_EINVAL, "truncated variable data");
      if (field[vli] >= 0) {
        if (cnt != (size_t)np) return fail(NMG_EMESH, "variable size differs from n^3");
        from_le(b.data() + pos, cnt, u + ((size_t)e * NMG_NFIELDS + field[vli]) * np);
      }
      pos += cnt * 8;
      if (pos < b.size() && b[pos] == '\n') pos++;
    }
    if (!seen[e]) nseen++;
    seen[e] = 1;
  }
  if (nseen != m->nelem) return fail(NMG_EMESH, "the file does not hold every element");
  return NMG_OK;
}

int nmg_checkpoint_write(nmg_ctx *c, const nmg_mesh *m, const char *path,
                         const char *const *names) {
  if (!c || !m) return fail(NMG_EINVAL, "nmg_checkpoint_write: null argument");
  std::vector<double> u((size_t)nmg_state_size(c));
  int rc = nmg_get_state(c, u.data());
  if (rc) return fail(rc, std::string("nmg_get_state: ") + nmg_last_error(c));
  return nmg_checkpoint_write_host(m, u.data(), path, names);
}

int nmg_checkpoint_read(nmg_ctx *c, const nmg_mesh *m, const char *path,
                        const char *const *names) {
  if (!c || !m) return fail(NMG_EINVAL, "nmg_checkpoint_read: null argument");
  if (nmg_state_size(c) != m->nelem * NMG_NFIELDS * (int64_t)m->n * m->n * m->n)
    return fail(NMG_EINVAL, "nmg_checkpoint_read: mesh and context differ");
  std::vector<double> u((size_t)nmg_state_size(c));
  int rc = nmg_checkpoint_read_host(m, path, u.data(), names);
  if (rc) return rc;
  rc = nmg_set_state(c, u.data());
  if (rc) return fail(rc, std::string("nmg_set_state: ") + nmg_last_error(c));
  return NMG_OK;
}

}  // extern "C"
