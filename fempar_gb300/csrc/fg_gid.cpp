// fg_gid.cpp -- reader of FEMPAR's GiD problem-type mesh files (<dir>/<prefix>.mesh), the
// input of the mesh-data-files route (Sources/Lib/Geometry/Mesh/mesh.f90:337-504):
//
//   MESH dimension 3 order O types T elements NC vertices NV vefs NB
//   coordinates            id x y z             ... end coordinates
//   elements               id nnode v1..vn set geo   ... end elements
//   vefs                   id nnodb v1..vk set geo   ... end vefs
//
// Sections are found by the first five characters of a line, as the reference does.  With
// order 0 ("c order", GiD's vertex order) the vertices of every hexahedron are reordered
// to the lexicographic local order by (1,2,4,3,5,6,8,7) (mesh.f90:52, :458-485).  The arrays
// then go to fg_mesh_create_unstructured, which validates every id.
#include <cerrno>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "fg_internal.h"

using fg::set_error;

namespace {

struct Lines {
  const char* p;
  const char* end;
  // next line [b, e) without the newline; false at the end of the buffer
  bool next(const char*& b, const char*& e) {
    if (p >= end) return false;
    b = p;
    const char* nl = static_cast<const char*>(memchr(p, '\n', (size_t)(end - p)));
    e = nl ? nl : end;
    p = nl ? nl + 1 : end;
    return true;
  }
};

bool starts(const char* b, const char* e, const char* key) {
  const size_t n = strlen(key);
  return (size_t)(e - b) >= n && memcmp(b, key, n) == 0;
}

// integers / doubles of one line, in order
bool parse_ints(const char* b, const char* e, std::vector<long long>& out) {
  out.clear();
  std::string s(b, e);
  const char* q = s.c_str();
  while (true) {
    while (*q == ' ' || *q == '\t' || *q == '\r') ++q;
    if (!*q) return true;
    char* r = nullptr;
    errno = 0;
    long long v = strtoll(q, &r, 10);
    if (r == q || errno) return false;
    out.push_back(v);
    q = r;
  }
}

}  // namespace

extern "C" fg_status fg_mesh_read_gid(fg_ctx* ctx, const char* dir_path, const char* prefix, fg_mesh** out) {
  if (!ctx || !dir_path || !prefix || !out) {
    set_error("bad argument: ctx/dir_path/prefix/out");
    return FG_ERR_BADARG;
  }
  *out = nullptr;
  const std::string path = std::string(dir_path) + "/" + prefix + ".mesh";
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) {
    set_error("cannot open %s", path.c_str());
    return FG_ERR_BADARG;
  }
  std::string buf;
  {
    char tmp[1 << 16];
    size_t n;
    while ((n = fread(tmp, 1, sizeof(tmp), f)) > 0) buf.append(tmp, n);
    fclose(f);
  }
  Lines L{buf.data(), buf.data() + buf.size()};
  const char *b, *e;
  if (!L.next(b, e) || !starts(b, e, "MESH")) {
    set_error("%s: no MESH header", path.c_str());
    return FG_ERR_BADARG;
  }
  long long dim = -1, order = -1, nelem = -1, npoin = -1, nboun = -1;
  {
    std::string h(b, e);
    const char* keys[] = {"dimension", "order", "elements", "vertices", "vefs"};
    long long* vals[] = {&dim, &order, &nelem, &npoin, &nboun};
    for (int k = 0; k < 5; ++k) {
      size_t at = h.find(keys[k]);
      if (at == std::string::npos) continue;
      *vals[k] = strtoll(h.c_str() + at + strlen(keys[k]), nullptr, 10);
    }
  }
  if (dim != 3) {
    set_error("%s: dimension %lld (only 3D hexahedral meshes are built on the device)", path.c_str(), dim);
    return FG_ERR_UNSUPPORTED;
  }
  if (nelem < 1 || npoin < 1 || nboun < 0) {
    set_error("%s: bad header counts", path.c_str());
    return FG_ERR_BADARG;
  }
  std::vector<double> xyz((size_t)npoin * 3, 0.0);
  std::vector<int32_t> cells((size_t)nelem * 8, 0);
  std::vector<std::vector<int32_t>> bv((size_t)nboun);
  std::vector<int32_t> bset((size_t)nboun, 0);
  std::vector<long long> tok;
  int section = 0;  // 1 coordinates, 2 elements, 3 vefs
  while (L.next(b, e)) {
    if (section == 0) {
      if (starts(b, e, "coord")) section = 1;
      else if (starts(b, e, "eleme")) section = 2;
      else if (starts(b, e, "vefs")) section = 3;
      continue;
    }
    if ((section == 1 && starts(b, e, "end c")) || (section == 2 && starts(b, e, "end e")) ||
        (section == 3 && starts(b, e, "end v"))) {
      section = 0;
      continue;
    }
    if (section == 1) {
      std::string s(b, e);
      char* r = nullptr;
      long long id = strtoll(s.c_str(), &r, 10);
      if (id < 1 || id > npoin) { set_error("%s: vertex id %lld", path.c_str(), id); return FG_ERR_BADARG; }
      for (int d = 0; d < 3; ++d) xyz[(size_t)(id - 1) * 3 + d] = strtod(r, &r);
    } else {
      if (!parse_ints(b, e, tok)) { set_error("%s: bad line", path.c_str()); return FG_ERR_BADARG; }
      if (tok.empty()) continue;
      if (tok.size() < 2) { set_error("%s: short line", path.c_str()); return FG_ERR_BADARG; }
      const long long id = tok[0], nn = tok[1];
      if ((long long)tok.size() < 2 + nn + 2) { set_error("%s: short line of entity %lld", path.c_str(), id); return FG_ERR_BADARG; }
      if (section == 2) {
        if (id < 1 || id > nelem) { set_error("%s: element id %lld", path.c_str(), id); return FG_ERR_BADARG; }
        if (nn != 8) { set_error("%s: element %lld has %lld vertices (hexahedra only)", path.c_str(), id, nn); return FG_ERR_UNSUPPORTED; }
        for (int k = 0; k < 8; ++k) cells[(size_t)(id - 1) * 8 + k] = (int32_t)tok[2 + k];
      } else {
        if (id < 1 || id > nboun) { set_error("%s: vef id %lld", path.c_str(), id); return FG_ERR_BADARG; }
        bv[id - 1].assign(tok.begin() + 2, tok.begin() + 2 + nn);
        bset[id - 1] = (int32_t)tok[2 + nn];
      }
    }
  }
  if (order == 0) {
    static const int permu[8] = {1, 2, 4, 3, 5, 6, 8, 7};
    for (long long c = 0; c < nelem; ++c) {
      int32_t t[8];
      for (int k = 0; k < 8; ++k) t[k] = cells[(size_t)c * 8 + permu[k] - 1];
      for (int k = 0; k < 8; ++k) cells[(size_t)c * 8 + k] = t[k];
    }
  }
  std::vector<int64_t> bptr((size_t)nboun + 1, 0);
  std::vector<int32_t> bverts;
  for (long long i = 0; i < nboun; ++i) {
    bverts.insert(bverts.end(), bv[i].begin(), bv[i].end());
    bptr[i + 1] = (int64_t)bverts.size();
  }
  return fg_mesh_create_unstructured(ctx, npoin, xyz.data(), nelem, cells.data(), nboun, bptr.data(),
                                     bverts.empty() ? nullptr : bverts.data(), bset.data(), out);
}
