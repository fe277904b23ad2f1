// Host mesh preprocessing of the typhon_gb300 library (no GPU).
//
// Builds the ty_mesh_desc arrays of include/typhon_gpu.h from an element mesh the way
// Typhon prepares a grid, so that face numbering, orientation, colours, ghost cells and
// every geometric value come out as Typhon computes them:
//   faces of each element, created cell by cell   CFDTOOLS/Mesh/create_facevtex.f90:60-210
//   interior faces first, boundary faces reversed  CFDTOOLS/Mesh/MESHCONNECT.f90:538-598
//   boundary marks matched to faces                CFDTOOLS/Mesh/seek_bcface_face.f90 (face
//                                                  elements), seek_bcface_vtex.f90 (vertices)
//   face/cell geometry                             CFDTOOLS/Mesh/MESHGEOM.f90:37-330
//   greedy first-fit face colouring                CFDTOOLS/Base/COLOR.f90:55-81
//   ghost cells, periodic partners                 SOURCE/ZONE/init_connect_grid.f90:60-246,
//                                                  SOURCE/ZONE/init_ustboco_ghostcell.f90:44-80,
//                                                  init_ustboco_ghostface.f90 (TY_BC_HEAT)
// Data structures differ from Typhon's (hash maps instead of vertex->face scans, a spatial
// hash for periodic matching) so that meshes of millions of cells preprocess in seconds.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/typhon_gpu.h"
#include "internal.hpp"

namespace {

struct V3 { double x, y, z; };
inline V3 mk(double a, double b, double c) { return V3{a, b, c}; }
inline V3 add(V3 a, V3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 sub(V3 a, V3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 scl(double s, V3 a) { return mk(s * a.x, s * a.y, s * a.z); }
inline V3 dvd(V3 a, double s) { return mk(a.x / s, a.y / s, a.z / s); }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double norm(V3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
inline V3 cross(V3 a, V3 b) { return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }

int elem_nv(int t) {
  switch (t) {
    case 2: return 2;     // BAR2
    case 13: return 3;    // TRI3
    case 24: return 4;    // QUAD4
    case 101: return 4;   // TETRA4
    case 131: return 6;   // PENTA6
    case 141: return 8;   // HEXA8
  }
  return 0;
}
int elem_dim(int t) {
  switch (t) {
    case 2: return 1;
    case 13: case 24: return 2;
    case 101: case 131: case 141: return 3;
  }
  return 0;
}

struct Section { int type; std::vector<int> ielem, vtex; };
struct Mark { std::string family; std::vector<int> tags; bool vertex = false; };
struct BcIn {
  std::string family, partner;
  int kind;
  V3 trans, wallvel;
  bool rot = false;     // periodic by rotation: centre, unit axis, angle (radians) to the partner
  V3 rc{0, 0, 0}, ra{0, 0, 1};
  double ang = 0.0;
};

// calc_rot (CFDTOOLS/Math/VEC3D.f90:652-674): row-major rotation about the unit axis a by
// angle; the same operations and order as the oracle's
void calc_rot(V3 a, double angle, double* M) {
  const double costh = std::cos(angle), sinth = std::sin(angle);
  const double ax[3] = {a.x, a.y, a.z};
  M[0] = costh; M[4] = costh; M[8] = costh;
  M[1] = -a.z * sinth; M[2] = +a.y * sinth;
  M[3] = +a.z * sinth; M[5] = -a.x * sinth;
  M[6] = -a.y * sinth; M[7] = +a.x * sinth;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) M[3 * i + j] = M[3 * i + j] + (1.0 - costh) * ax[i] * ax[j];
}
V3 rot_apply(const double* M, V3 v) {
  return mk(M[0] * v.x + M[1] * v.y + M[2] * v.z, M[3] * v.x + M[4] * v.y + M[5] * v.z,
            M[6] * v.x + M[7] * v.y + M[8] * v.z);
}

std::string upper(std::string s) {
  for (auto& c : s) c = (char)toupper((unsigned char)c);
  return s;
}

// Faces are identified by their sorted vertex list (up to 4 vertices).
struct FaceKey {
  std::array<int, 4> v;
  bool operator==(const FaceKey& o) const { return v == o.v; }
};

// Face lookup during face creation: the faces are bucketed by their smallest vertex, each
// bucket a contiguous run of slots sized beforehand from the element faces (each face is
// visited at most twice, so a bucket never outgrows the count).  Neighbouring cells share
// vertices, and vertices are numbered with the mesh, so the lookups of a sweep over the cells
// stay in a few cache lines instead of hashing across the whole table.
class FaceBuckets {
 public:
  // count[v]: element faces whose smallest vertex is v (vertices 1..nv)
  explicit FaceBuckets(const std::vector<int>& count) : start_(count.size() + 1, 0), fill_(count.size(), 0) {
    for (size_t v = 0; v < count.size(); ++v) start_[v + 1] = start_[v] + count[v];
    slots_.resize(start_.back());
  }
  // the face id of key, or -1 after inserting key with id `fresh`
  int find_or_insert(const FaceKey& key, int fresh) {
    const int v = key.v[0];
    Slot* b = slots_.data() + start_[v];
    for (int i = 0; i < fill_[v]; ++i)
      if (b[i].a == key.v[1] && b[i].b == key.v[2] && b[i].c == key.v[3]) return b[i].id;
    b[fill_[v]++] = Slot{key.v[1], key.v[2], key.v[3], fresh};
    return -1;
  }
  // the face id of key, or -1
  int find(const FaceKey& key) const {
    const int v = key.v[0];
    if (v < 0 || v >= (int)fill_.size()) return -1;
    const Slot* b = slots_.data() + start_[v];
    for (int i = 0; i < fill_[v]; ++i)
      if (b[i].a == key.v[1] && b[i].b == key.v[2] && b[i].c == key.v[3]) return b[i].id;
    return -1;
  }
  // every stored id f replaced by newidx[f]
  void remap(const std::vector<int>& newidx) {
    for (size_t v = 0; v < fill_.size(); ++v)
      for (int i = 0; i < fill_[v]; ++i) {
        Slot& sl = slots_[start_[v] + i];
        sl.id = newidx[sl.id];
      }
  }

 private:
  struct Slot {
    int a, b, c, id;  // the other three sorted vertices (0 padded) and the face id
  };
  std::vector<size_t> start_;
  std::vector<int> fill_;
  std::vector<Slot> slots_;
};
// the n (2..4) vertices of a face in increasing order, zero padded
FaceKey key_of(const int* f, int n) {
  FaceKey k;
  k.v = {0, 0, 0, 0};
  for (int i = 0; i < n && i < 4; ++i) {  // insertion sort of at most four entries
    int x = f[i], j = i;
    for (; j > 0 && k.v[j - 1] > x; --j) k.v[j] = k.v[j - 1];
    k.v[j] = x;
  }
  return k;
}

}  // namespace

struct ty_umesh {
  std::vector<V3> nodes;
  std::vector<Section> sections;
  std::vector<Mark> marks;
  std::vector<BcIn> bcs;
  bool built = false;
  int dim = 0, ncell_int = 0, ncell = 0, nface_int = 0, nface = 0;
  std::vector<int32_t> facecell;          // [2*nface], 1-based, column-major
  std::vector<int32_t> facevtex;          // [4*nface], 1-based, 0 padded
  std::vector<V3> fnormal, fcentre, ccentre;  // exported as [n][3] doubles (V3 holds three)
  std::vector<double> fsurf, cvol, fwallvel;
  std::vector<int32_t> fcolor, fbc, fpartner, ffamily;
  std::vector<double> frot;               // [nface][9] rotation into each face's frame
  bool has_rot = false;
};

extern "C" {

int ty_umesh_new(ty_umesh** out) {
  if (!out) return TY_ERR_ARG;
  *out = new ty_umesh();
  return TY_OK;
}
int ty_umesh_free(ty_umesh* um) {
  delete um;
  return TY_OK;
}
int ty_umesh_set_nodes(ty_umesh* um, int32_t n, const double* xyz) {
  if (!um || n < 0 || (n && !xyz)) return TY_ERR_ARG;
  um->nodes.resize(n);
  for (int i = 0; i < n; ++i) um->nodes[i] = mk(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
  return TY_OK;
}
int ty_umesh_add_section(ty_umesh* um, int32_t type, int32_t nelem, const int32_t* ielem,
                         const int32_t* vtex) {
  if (!um || nelem < 0 || elem_nv(type) == 0 || (nelem && (!ielem || !vtex))) return TY_ERR_ARG;
  Section s;
  s.type = type;
  s.ielem.assign(ielem, ielem + nelem);
  s.vtex.assign(vtex, vtex + (size_t)nelem * elem_nv(type));
  um->sections.push_back(std::move(s));
  return TY_OK;
}
int ty_umesh_add_mark(ty_umesh* um, const char* family, int32_t ntag, const int32_t* tags) {
  if (!um || !family || ntag < 0 || (ntag && !tags)) return TY_ERR_ARG;
  Mark m;
  m.family = family;
  m.tags.assign(tags, tags + ntag);
  um->marks.push_back(std::move(m));
  return TY_OK;
}
int ty_umesh_add_vertex_mark(ty_umesh* um, const char* family, int32_t ntag, const int32_t* tags) {
  int rc = ty_umesh_add_mark(um, family, ntag, tags);
  if (rc == TY_OK) um->marks.back().vertex = true;
  return rc;
}
int ty_umesh_add_bc(ty_umesh* um, const char* family, int32_t kind, const char* partner,
                    const double* t3, const double* w3) {
  if (!um || !family || kind < TY_BC_PERIODIC || kind > TY_BC_OUTLET_SUP) return TY_ERR_ARG;
  BcIn b;
  b.family = upper(family);
  b.partner = partner ? upper(partner) : "";
  b.kind = kind;
  b.trans = t3 ? mk(t3[0], t3[1], t3[2]) : mk(0, 0, 0);
  b.wallvel = w3 ? mk(w3[0], w3[1], w3[2]) : mk(0, 0, 0);
  um->bcs.push_back(b);
  return TY_OK;
}

int ty_umesh_build(ty_umesh* um, int32_t dim) {
  if (!um || (dim != 2 && dim != 3)) return TY_ERR_ARG;
  auto fail = [&](const char* msg) { tyi::set_error(msg); return TY_ERR_MESH; };
  um->dim = dim;
  const int nvtex = (int)um->nodes.size();
  int maxdim = 0;
  for (auto& s : um->sections) maxdim = std::max(maxdim, elem_dim(s.type));
  int ncell_int = 0;
  for (auto& s : um->sections)
    if (elem_dim(s.type) == maxdim) ncell_int += (int)s.ielem.size();

  // ---- faces in creation order ----
  std::vector<int> fv;        // 4 per face, creation order
  std::vector<int> fnv;       // vertex count per face
  std::vector<int> c1, c2;    // 1-based cells, 0 = none
  size_t nface_max = 0;  // faces created at most: one per element face
  for (auto& s : um->sections) {
    if (elem_dim(s.type) != maxdim) continue;
    const int per = s.type == 13 ? 3 : s.type == 24 ? 4 : s.type == 101 ? 4 : s.type == 131 ? 5 : 6;
    nface_max += (size_t)per * s.ielem.size();
  }
  static const int tri[3][2] = {{1, 2}, {2, 3}, {3, 1}};
  static const int quad[4][2] = {{1, 2}, {2, 3}, {3, 4}, {4, 1}};
  static const int tet[4][3] = {{1, 3, 2}, {1, 2, 4}, {2, 3, 4}, {3, 1, 4}};
  static const int hexa[6][4] = {{1, 2, 3, 4}, {1, 2, 6, 5}, {5, 6, 7, 8},
                                 {4, 3, 7, 8}, {1, 4, 8, 5}, {2, 3, 7, 6}};
  static const int pr_t1[3] = {1, 2, 3}, pr_t2[3] = {4, 5, 6};
  static const int pr_q1[4] = {1, 3, 6, 4}, pr_q2[4] = {1, 2, 5, 4}, pr_q3[4] = {2, 3, 6, 5};
  // the faces of one element in creation order (create_facevtex.f90); fn(local vertices, n)
  // returns false to stop
  auto for_each_face = [&](int type, auto&& fn) -> int {  // 1 done, 0 stopped, -1 unknown type
    switch (type) {
      case 13: for (int k = 0; k < 3; ++k) if (!fn(tri[k], 2)) return 0; return 1;
      case 24: for (int k = 0; k < 4; ++k) if (!fn(quad[k], 2)) return 0; return 1;
      case 101: for (int k = 0; k < 4; ++k) if (!fn(tet[k], 3)) return 0; return 1;
      case 131:
        return (fn(pr_t1, 3) && fn(pr_t2, 3) && fn(pr_q1, 4) && fn(pr_q2, 4) && fn(pr_q3, 4)) ? 1 : 0;
      case 141: for (int k = 0; k < 6; ++k) if (!fn(hexa[k], 4)) return 0; return 1;
      default: return -1;
    }
  };
  // bucket sizes: element faces per smallest vertex (faces with a vertex out of range are
  // rejected in the creation pass below)
  std::vector<int> per_vertex((size_t)nvtex + 1, 0);
  for (auto& s : um->sections) {
    if (elem_dim(s.type) != maxdim) continue;
    const int nv = elem_nv(s.type);
    for (size_t ic = 0; ic < s.ielem.size(); ++ic) {
      const int* e = &s.vtex[ic * nv];
      if (for_each_face(s.type, [&](const int* loc, int n) {
            int m = e[loc[0] - 1];
            for (int k = 1; k < n; ++k) m = std::min(m, e[loc[k] - 1]);
            if (m >= 1 && m <= nvtex) ++per_vertex[m];
            return true;
          }) < 0)
        return fail("unsupported element type");
    }
  }
  FaceBuckets lookup(per_vertex);
  fv.reserve(4 * nface_max / 2 + 16);
  fnv.reserve(nface_max / 2 + 4);
  c1.reserve(nface_max / 2 + 4);
  c2.reserve(nface_max / 2 + 4);
  for (auto& s : um->sections) {
    if (elem_dim(s.type) != maxdim) continue;
    const int nv = elem_nv(s.type);
    for (size_t ic = 0; ic < s.ielem.size(); ++ic) {
      const int icell = s.ielem[ic];
      const int* e = &s.vtex[ic * nv];
      auto create = [&](const int* loc, int n) -> bool {
        int f[4] = {0, 0, 0, 0};
        for (int k = 0; k < n; ++k) {
          f[k] = e[loc[k] - 1];
          if (f[k] < 1 || f[k] > nvtex) return false;
        }
        const FaceKey key = key_of(f, n);
        const int id = lookup.find_or_insert(key, (int)c1.size());
        if (id < 0) {
          for (int k = 0; k < 4; ++k) fv.push_back(f[k]);
          fnv.push_back(n);
          c1.push_back(icell);
          c2.push_back(0);
        } else {
          if (c2[id] != 0) return false;
          c2[id] = icell;
        }
        return true;
      };
      const int r = for_each_face(s.type, create);
      if (r < 0) return fail("unsupported element type");
      if (r == 0) return fail("bad connectivity (vertex out of range or 3 cells on a face)");
    }
  }
  const int nface = (int)c1.size();

  // ---- reorder: interior faces first in creation order, boundary faces reversed ----
  std::vector<int> newidx(nface);
  int nfi = 0, nfl = 0;
  for (int f = 0; f < nface; ++f) {
    if (c2[f] == 0) { ++nfl; newidx[f] = nface - nfl; }
    else newidx[f] = nfi++;
  }
  std::vector<int> F1(nface), F2(nface), FV(4 * (size_t)nface), FN(nface);
  for (int f = 0; f < nface; ++f) {
    int n = newidx[f];
    F1[n] = c1[f]; F2[n] = c2[f]; FN[n] = fnv[f];
    for (int k = 0; k < 4; ++k) FV[4 * (size_t)n + k] = fv[4 * (size_t)f + k];
  }
  lookup.remap(newidx);

  // ---- boundary marks -> boundary faces (mark order) ----
  struct Boco { std::string family; std::vector<int> iface; int kind = 0; int def = -1; double rlink = 0;
                std::vector<int> partner; };
  std::vector<Boco> bocos;
  {
    std::unordered_map<int, std::pair<int, int>> face_elem;  // element number -> (section, index)
    for (size_t si = 0; si < um->sections.size(); ++si) {
      auto& s = um->sections[si];
      if (elem_dim(s.type) != maxdim - 1) continue;
      for (size_t i = 0; i < s.ielem.size(); ++i) face_elem.emplace(s.ielem[i], std::make_pair((int)si, (int)i));
    }
    for (auto& mkr : um->marks) {
      Boco b;
      b.family = upper(mkr.family);
      if (mkr.vertex) {  // every vertex of the boundary face in the list (seek_bcface_vtex.f90:38-45)
        std::vector<int> sorted(mkr.tags);
        std::sort(sorted.begin(), sorted.end());
        for (int f = nfi; f < nface; ++f) {
          bool all = true;
          for (int k = 0; k < 4 && all; ++k) {
            const int v = FV[4 * (size_t)f + k];
            all = v == 0 || std::binary_search(sorted.begin(), sorted.end(), v);
          }
          if (all) b.iface.push_back(f);
        }
        if (!b.iface.empty()) bocos.push_back(std::move(b));
        continue;
      }
      for (int tag : mkr.tags) {
        auto it = face_elem.find(tag);
        if (it == face_elem.end()) continue;
        auto& s = um->sections[it->second.first];
        int nv = elem_nv(s.type);
        const int fk = lookup.find(key_of(&s.vtex[(size_t)it->second.second * nv], nv));
        if (fk >= nfi) b.iface.push_back(fk);
      }
      if (!b.iface.empty()) bocos.push_back(std::move(b));
    }
    size_t nb = 0;
    for (auto& b : bocos) nb += b.iface.size();
    if ((int)nb != nfl) return fail("tagged faces do not match the boundary faces");
  }
  const int ncell = ncell_int + nfl;

  // ---- geometry (operation order of MESHGEOM.f90) ----
  std::vector<V3> fn(nface), fc(nface), cc(ncell, mk(0, 0, 0));
  std::vector<double> fs(nface), cv(ncell, 0.0);
  auto X = [&](int iv) { return um->nodes[iv - 1]; };
  for (int f = 0; f < nface; ++f) {
    const int* v = &FV[4 * (size_t)f];
    if (dim == 2) {
      if (FN[f] != 2) return fail("2D meshes need 2-vertex faces");
      V3 nrm = cross(mk(0., 0., 1.), sub(X(v[1]), X(v[0])));
      double s = norm(nrm);
      fn[f] = dvd(nrm, s);
      fs[f] = s;
      fc[f] = scl(0.5, add(X(v[0]), X(v[1])));
    } else if (FN[f] == 3) {
      V3 a = X(v[0]), b = X(v[1]), c = X(v[2]);
      V3 nrm = scl(0.5, cross(sub(b, a), sub(c, a)));
      double s = norm(nrm);
      fn[f] = dvd(nrm, s);
      fs[f] = s;
      fc[f] = dvd(add(add(a, b), c), 3.0);
    } else if (FN[f] == 4) {
      V3 a = X(v[0]), b = X(v[1]), c = X(v[2]), d = X(v[3]);
      V3 nrm = scl(0.5, cross(sub(b, a), sub(c, a)));
      double s1 = norm(nrm);
      V3 cg1 = dvd(add(add(a, b), c), 3.0);
      V3 pt = scl(0.5, cross(sub(c, a), sub(d, a)));
      double s2 = norm(pt);
      V3 cg2 = dvd(add(add(a, c), d), 3.0);
      nrm = add(nrm, pt);
      double s = norm(nrm);
      fn[f] = dvd(nrm, s);
      fs[f] = s;
      fc[f] = dvd(add(scl(s1, cg1), scl(s2, cg2)), s1 + s2);
    } else {
      return fail("faces with 3 or 4 vertices expected in 3D");
    }
  }
  {
    std::vector<V3> mid(ncell_int, mk(0, 0, 0));
    std::vector<int> nb(ncell_int, 0);
    for (int f = 0; f < nface; ++f) {
      int a = F1[f] - 1;
      mid[a] = add(mid[a], fc[f]);
      nb[a]++;
      if (F2[f] > 0 && F2[f] <= ncell_int) {
        int b = F2[f] - 1;
        mid[b] = add(mid[b], fc[f]);
        nb[b]++;
      }
    }
    for (int c = 0; c < ncell_int; ++c) mid[c] = dvd(mid[c], (double)nb[c]);
    const double kcg = dim == 2 ? 1.0 / 3.0 : 1.0 / 4.0;
    const double kvol = dim == 2 ? 1.0 / 2.0 : 1.0 / 3.0;
    auto elem = [&](V3 vK, int f, V3& cg, double& vol) {
      V3 vKH = sub(fc[f], vK);
      double h = std::fabs(dot(vKH, fn[f]));
      cg = sub(fc[f], scl(kcg, vKH));
      vol = kvol * h * fs[f];
    };
    for (int f = 0; f < nface; ++f) {
      V3 cg; double vol;
      int a = F1[f] - 1;
      elem(mid[a], f, cg, vol);
      cc[a] = add(cc[a], scl(vol, cg));
      cv[a] = cv[a] + vol;
      if (F2[f] > 0 && F2[f] <= ncell_int) {
        int b = F2[f] - 1;
        elem(mid[b], f, cg, vol);
        cc[b] = add(cc[b], scl(vol, cg));
        cv[b] = cv[b] + vol;
      }
    }
    for (int c = 0; c < ncell_int; ++c) {
      if (!(cv[c] > 0.0)) return fail("degenerate cell (zero volume)");
      cc[c] = dvd(cc[c], cv[c]);
    }
  }
  for (int f = 0; f < nface; ++f)
    if (F2[f] != 0 && F1[f] > F2[f]) std::swap(F1[f], F2[f]);
  for (int f = 0; f < nface; ++f) {
    V3 v12 = F2[f] != 0 ? sub(cc[F2[f] - 1], cc[F1[f] - 1]) : sub(fc[f], cc[F1[f] - 1]);
    if (dot(v12, fn[f]) < 0.0) fn[f] = mk(-fn[f].x, -fn[f].y, -fn[f].z);
  }

  // ---- greedy colouring: the first colour free at both cells (boundary: one cell) ----
  std::vector<int> color(nface);
  bool coloured = false;
  {  // colours of each cell as a bit mask (the first free colour is the lowest clear bit)
    std::vector<uint64_t> used(ncell, 0);
    int ncolor = 0;
    coloured = true;
    for (int f = 0; f < nface && coloured; ++f) {
      const int a = F1[f] - 1;
      const int b = (F2[f] == 0 || F2[f] > ncell) ? a : F2[f] - 1;
      const uint64_t u = used[a] | used[b];
      int chosen = 0;
      while (chosen < ncolor && ((u >> chosen) & 1u)) ++chosen;
      if (chosen == ncolor) ++ncolor;
      if (ncolor > 64) { coloured = false; break; }  // more colours than bits: the general form
      color[f] = chosen;
      used[a] |= 1ull << chosen;
      used[b] |= 1ull << chosen;
    }
  }
  if (!coloured) {
    std::vector<std::vector<int>> vcol(ncell);
    int ncolor = 0;
    for (int f = 0; f < nface; ++f) {
      int a = F1[f] - 1;
      int b = (F2[f] == 0 || F2[f] > ncell) ? a : F2[f] - 1;
      int chosen = -1;
      for (int ic = 0; ic < ncolor && chosen < 0; ++ic) {
        bool used = std::find(vcol[a].begin(), vcol[a].end(), ic) != vcol[a].end() ||
                    std::find(vcol[b].begin(), vcol[b].end(), ic) != vcol[b].end();
        if (!used) chosen = ic;
      }
      if (chosen < 0) chosen = ncolor++;
      color[f] = chosen;
      vcol[a].push_back(chosen);
      vcol[b].push_back(chosen);
    }
  }

  // ---- ghost cells: physical boundaries first, then periodic connections ----
  std::vector<int> fbc(nface, TY_BC_INTERIOR), fpart(nface, 0), ffam(nface, -1);
  // rotation into each face's frame (identity), stored only when a family is rotational
  bool any_rot = false;
  for (const auto& b : um->bcs) any_rot = any_rot || b.rot;
  std::vector<double> frot(any_rot ? 9 * (size_t)nface : 0, 0.0);
  if (any_rot)
    for (int f = 0; f < nface; ++f) frot[9 * (size_t)f] = frot[9 * (size_t)f + 4] = frot[9 * (size_t)f + 8] = 1.0;
  std::vector<double> fwall(3 * (size_t)nface, 0.0);
  int nlim = 0;
  for (auto& b : bocos) {
    for (size_t i = 0; i < um->bcs.size(); ++i)
      if (um->bcs[i].kind != TY_BC_PERIODIC && um->bcs[i].family == b.family) { b.def = (int)i; break; }
    if (b.def >= 0) {
      const BcIn& d = um->bcs[b.def];
      b.kind = d.kind;
      for (int f : b.iface) {
        ++nlim;
        int a = F1[f] - 1, g = ncell_int + nlim - 1;
        F2[f] = g + 1;
        fbc[f] = d.kind;
        ffam[f] = b.def;
        fwall[3 * (size_t)f] = d.wallvel.x; fwall[3 * (size_t)f + 1] = d.wallvel.y; fwall[3 * (size_t)f + 2] = d.wallvel.z;
        cv[g] = cv[a];
        if (d.kind == TY_BC_HEAT || d.kind >= TY_BC_INLET_SUB) {  // ghost face (init_ustboco_ghostface.f90:46-56)
          cv[g] = 0.0;
          cc[g] = fc[f];
        } else if (d.kind == TY_BC_SYMMETRY) {
          V3 n = fn[f], gc = cc[a];
          cc[g] = add(gc, scl(2.0 * dot(sub(fc[f], gc), n), n));
        } else {
          cc[g] = sub(scl(2.0, fc[f]), cc[a]);
        }
      }
      continue;
    }
    for (size_t i = 0; i < um->bcs.size(); ++i) {
      if (um->bcs[i].kind != TY_BC_PERIODIC) continue;
      if (um->bcs[i].family == b.family) { b.def = (int)i; b.rlink = 1.0; break; }
      if (um->bcs[i].partner == b.family) { b.def = (int)i; b.rlink = -1.0; break; }
    }
    if (b.def < 0) return fail("a boundary family has no definition");
    b.kind = TY_BC_PERIODIC;
  }
  for (auto& b : bocos) {
    if (b.kind != TY_BC_PERIODIC) continue;
    const BcIn& d = um->bcs[b.def];
    Boco* b2 = nullptr;
    for (auto& o : bocos)
      if (o.kind == TY_BC_PERIODIC && o.def == b.def && o.rlink * b.rlink < 0) {
        if (b2) return fail("too many matching periodic families");
        b2 = &o;
      }
    if (!b2 || b2->iface.size() != b.iface.size()) return fail("no matching periodic family");
    // nearest partner face centre to each translated face centre (spatial hash, ties to the
    // lowest index as in matching_index)
    const size_t nf = b.iface.size();
    double h = std::numeric_limits<double>::max();
    for (int f : b2->iface) h = std::min(h, std::sqrt(fs[f]));
    if (!(h > 0.0)) h = 1.0;
    auto cell_of = [&](V3 p) {
      return std::array<long long, 3>{(long long)std::floor(p.x / h), (long long)std::floor(p.y / h),
                                      (long long)std::floor(p.z / h)};
    };
    struct AH { size_t operator()(const std::array<long long, 3>& a) const {
      return (size_t)(a[0] * 73856093LL ^ a[1] * 19349663LL ^ a[2] * 83492791LL); } };
    std::unordered_map<std::array<long long, 3>, std::vector<int>, AH> grid;
    for (size_t k = 0; k < nf; ++k) grid[cell_of(fc[b2->iface[k]])].push_back((int)k);
    b.partner.resize(nf);
    double Mloc[9], Mvec[9];  // transloc_per (rlink * angle) and transvec_per (-rlink * angle)
    if (d.rot) {
      calc_rot(d.ra, b.rlink * d.ang, Mloc);
      calc_rot(d.ra, -b.rlink * d.ang, Mvec);
    }
    for (size_t k = 0; k < nf; ++k) {
      V3 p = fc[b.iface[k]];
      if (d.rot) p = add(rot_apply(Mloc, sub(p, d.rc)), d.rc);
      else p = add(p, scl(b.rlink, d.trans));
      auto c0 = cell_of(p);
      double best = std::numeric_limits<double>::max();
      int ib = -1;
      for (long long dx = -1; dx <= 1; ++dx)
        for (long long dy = -1; dy <= 1; ++dy)
          for (long long dz = -1; dz <= 1; ++dz) {
            auto it = grid.find({c0[0] + dx, c0[1] + dy, c0[2] + dz});
            if (it == grid.end()) continue;
            for (int j : it->second) {
              double dist = norm(sub(p, fc[b2->iface[j]]));
              if (dist < best || (dist == best && j < ib)) { best = dist; ib = j; }
            }
          }
      // matching_index (GRID_CONNECT.f90) takes the nearest face with no tolerance; the guard
      // allows for meshes written with single-precision-like coordinates (perrot2d.cgns: 3e-8)
      if (ib < 0 || !(best <= 1e-3 * h)) return fail("periodic faces do not match");
      b.partner[k] = b2->iface[ib];
    }
    for (int f : b.iface) {
      ++nlim;
      F2[f] = ncell_int + nlim;
    }
    for (size_t k = 0; k < nf; ++k) {
      int f = b.iface[k], fp = b.partner[k];
      int g = F2[f] - 1, icper = F1[fp] - 1;
      V3 dfc = sub(cc[icper], fc[fp]);
      if (d.rot) {  // init_connect_grid.f90:218-223: the face-to-cell vector rotated
        dfc = rot_apply(Mvec, dfc);
        for (int q = 0; q < 9; ++q) frot[9 * (size_t)f + q] = Mvec[q];
      }
      cv[g] = cv[icper];
      cc[g] = add(fc[f], dfc);
      fbc[f] = TY_BC_PERIODIC;
      ffam[f] = b.def;
      fpart[f] = fp + 1;
    }
  }
  for (int f = 0; f < nface; ++f)
    if (F2[f] == 0) return fail("boundary face without ghost cell");

  // ---- export ----
  um->ncell_int = ncell_int; um->ncell = ncell; um->nface_int = nfi; um->nface = nface;
  um->facecell.resize(2 * (size_t)nface);
  for (int f = 0; f < nface; ++f) { um->facecell[f] = F1[f]; um->facecell[nface + f] = F2[f]; }
  um->facevtex.assign(FV.begin(), FV.end());
  for (int f = 0; f < nface; ++f)
    for (int k = FN[f]; k < 4; ++k) um->facevtex[4 * (size_t)f + k] = 0;
  um->fnormal = std::move(fn);
  um->fcentre = std::move(fc);
  um->ccentre = std::move(cc);
  um->fsurf = std::move(fs);
  um->cvol = std::move(cv);
  um->fcolor = std::move(color);
  um->fbc = std::move(fbc);
  um->fpartner = std::move(fpart);
  um->fwallvel = std::move(fwall);
  um->ffamily = std::move(ffam);
  um->frot = std::move(frot);
  um->has_rot = any_rot;
  um->built = true;
  return TY_OK;
}

int ty_umesh_desc(const ty_umesh* um, ty_mesh_desc* d) {
  if (!um || !d || !um->built) return TY_ERR_STATE;
  d->dim = um->dim;
  d->ncell_int = um->ncell_int; d->ncell = um->ncell;
  d->nface_int = um->nface_int; d->nface = um->nface;
  d->facecell = um->facecell.data();
  static_assert(sizeof(V3) == 3 * sizeof(double), "V3 must be three packed doubles");
  d->face_normal = reinterpret_cast<const double*>(um->fnormal.data());
  d->face_surface = um->fsurf.data();
  d->face_centre = reinterpret_cast<const double*>(um->fcentre.data());
  d->cell_centre = reinterpret_cast<const double*>(um->ccentre.data());
  d->cell_volume = um->cvol.data();
  d->face_color = um->fcolor.data();
  d->face_bc = um->fbc.data();
  d->face_partner = um->fpartner.data();
  d->face_wallvel = um->fwallvel.data();
  return TY_OK;
}

int ty_umesh_set_rotation(ty_umesh* um, const char* family, const double* centre3, const double* axis3,
                          double angle_deg) {
  if (!um || !family || !centre3 || !axis3) return TY_ERR_ARG;
  const double an = std::sqrt(axis3[0] * axis3[0] + axis3[1] * axis3[1] + axis3[2] * axis3[2]);
  if (!(an > 0.0)) { tyi::set_error("ty_umesh_set_rotation: zero axis"); return TY_ERR_ARG; }
  for (auto& b : um->bcs)
    if (b.kind == TY_BC_PERIODIC && b.family == upper(family)) {
      b.rot = true;
      b.rc = mk(centre3[0], centre3[1], centre3[2]);
      b.ra = mk(axis3[0] / an, axis3[1] / an, axis3[2] / an);
      b.ang = angle_deg / 180.0 * 3.141592653589793238462643;  // def_mesh.f90:242-244
      um->built = false;
      return TY_OK;
    }
  tyi::set_error(std::string("ty_umesh_set_rotation: no periodic definition for family ") + family);
  return TY_ERR_ARG;
}

int ty_umesh_face_rotation(const ty_umesh* um, double* out) {
  if (!um || !out || !um->built) return TY_ERR_STATE;
  if (!um->has_rot) {  // the identity everywhere
    for (int f = 0; f < um->nface; ++f)
      for (int q = 0; q < 9; ++q) out[9 * (size_t)f + q] = (q % 4 == 0) ? 1.0 : 0.0;
    return 0;
  }
  std::memcpy(out, um->frot.data(), um->frot.size() * sizeof(double));
  return 1;
}

int ty_umesh_face_family(const ty_umesh* um, int32_t* out) {
  if (!um || !out || !um->built) return TY_ERR_STATE;
  std::memcpy(out, um->ffamily.data(), um->ffamily.size() * sizeof(int32_t));
  return TY_OK;
}

int ty_umesh_rcm_order(const ty_umesh* um, int32_t* order) {
  if (!um || !order || !um->built) return TY_ERR_STATE;
  int maxdim = 0;
  for (auto& s : um->sections) maxdim = std::max(maxdim, elem_dim(s.type));
  const int nci = um->ncell_int, nface = um->nface;
  // section and position of every cell
  std::vector<int> sec_of((size_t)nci + 1, -1), pos_of((size_t)nci + 1, -1);
  for (size_t si = 0; si < um->sections.size(); ++si) {
    const Section& s = um->sections[si];
    if (elem_dim(s.type) != maxdim) continue;
    for (size_t p = 0; p < s.ielem.size(); ++p) {
      const int id = s.ielem[p];
      if (id < 1 || id > nci) return TY_ERR_MESH;
      sec_of[id] = (int)si;
      pos_of[id] = (int)p;
    }
  }
  size_t off = 0;
  for (size_t si = 0; si < um->sections.size(); ++si) {
    const Section& s = um->sections[si];
    if (elem_dim(s.type) != maxdim) continue;
    const int m = (int)s.ielem.size();
    // adjacency of the section's cells through interior faces (CSR over positions)
    std::vector<int> deg(m, 0);
    for (int f = 0; f < nface; ++f) {
      const int a = um->facecell[f], b = um->facecell[nface + f];
      if (b < 1 || b > nci || a < 1 || a > nci) continue;
      if (sec_of[a] != (int)si || sec_of[b] != (int)si) continue;
      ++deg[pos_of[a]];
      ++deg[pos_of[b]];
    }
    std::vector<size_t> xadj((size_t)m + 1, 0);
    for (int p = 0; p < m; ++p) xadj[p + 1] = xadj[p] + deg[p];
    std::vector<int> adj(xadj[m]), fill(m, 0);
    for (int f = 0; f < nface; ++f) {
      const int a = um->facecell[f], b = um->facecell[nface + f];
      if (b < 1 || b > nci || a < 1 || a > nci) continue;
      if (sec_of[a] != (int)si || sec_of[b] != (int)si) continue;
      const int pa = pos_of[a], pb = pos_of[b];
      adj[xadj[pa] + fill[pa]++] = pb;
      adj[xadj[pb] + fill[pb]++] = pa;
    }
    // Cuthill-McKee from a pseudo-peripheral cell of each connected component (the
    // lowest-degree cell of the last level of a breadth-first search from the lowest-degree
    // unvisited cell), neighbours in increasing degree; then the whole order reversed
    std::vector<int> by_deg(m);
    for (int p = 0; p < m; ++p) by_deg[p] = p;
    std::stable_sort(by_deg.begin(), by_deg.end(), [&](int x, int y) { return deg[x] < deg[y]; });
    std::vector<char> seen(m, 0);
    std::vector<int> cm, level, mark(m, -1), nb;
    cm.reserve(m);
    size_t next_start = 0;
    int stamp = 0;
    while ((int)cm.size() < m) {
      while (seen[by_deg[next_start]]) ++next_start;
      int start = by_deg[next_start];
      // one breadth-first search to move the start to the far side of its component
      {
        ++stamp;
        level.assign(1, start);
        mark[start] = stamp;
        std::vector<int> last = level;
        while (!level.empty()) {
          last = level;
          std::vector<int> nxt;
          for (int u : level)
            for (size_t k = xadj[u]; k < xadj[u + 1]; ++k) {
              const int w = adj[k];
              if (mark[w] != stamp && !seen[w]) { mark[w] = stamp; nxt.push_back(w); }
            }
          level.swap(nxt);
        }
        for (int u : last)
          if (deg[u] < deg[start] || (deg[u] == deg[start] && u < start)) start = u;
      }
      size_t head = cm.size();
      cm.push_back(start);
      seen[start] = 1;
      while (head < cm.size()) {
        const int u = cm[head++];
        nb.clear();
        for (size_t k = xadj[u]; k < xadj[u + 1]; ++k)
          if (!seen[adj[k]]) { seen[adj[k]] = 1; nb.push_back(adj[k]); }
        std::stable_sort(nb.begin(), nb.end(), [&](int x, int y) { return deg[x] < deg[y]; });
        cm.insert(cm.end(), nb.begin(), nb.end());
      }
    }
    for (int k = 0; k < m; ++k) order[off + k] = cm[m - 1 - k];
    off += m;
  }
  return TY_OK;
}

int ty_umesh_facevtex(const ty_umesh* um, int32_t* out) {
  if (!um || !out || !um->built) return TY_ERR_STATE;
  std::memcpy(out, um->facevtex.data(), um->facevtex.size() * sizeof(int32_t));
  return TY_OK;
}

}  // extern "C"
