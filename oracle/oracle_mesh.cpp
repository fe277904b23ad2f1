// Typhon CPU oracle — mesh half.  TEST INFRASTRUCTURE ONLY (see oracle.hpp).
//
// Restates, in Typhon's loop order:
//   XBIN / TYPHON mesh reader      CFDTOOLS/FileFormat/internal/XBIN_IO.f90:86-135,
//                                  XBIN_DATA.f90:139-186, TYFMT_MESH.f90 (typhonread_*)
//   face creation                  CFDTOOLS/Mesh/create_facevtex.f90:15-220,
//                                  CFDTOOLS/Mesh/MESHCONNECT.f90:34-163 (ust_create_face,
//                                  scanface_vtexface, same_face)
//   face reordering                MESHCONNECT.f90:511-606 (reorder_ustconnect)
//   boundary marks -> faces        CFDTOOLS/Mesh/seek_bcface_face.f90, seek_bcface_vtex.f90
//   geometry                       CFDTOOLS/Mesh/MESHGEOM.f90:37-461
//   greedy face colouring          CFDTOOLS/Base/COLOR.f90:33-84
//   ghost cells and periodicity    SOURCE/ZONE/init_connect_grid.f90:60-246,
//                                  SOURCE/ZONE/init_ustboco_ghostcell.f90:30-84,
//                                  CFDTOOLS/Mesh/GRID_CONNECT.f90:120-150 (matching_index)
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <limits>

#include "oracle.hpp"

namespace ory {

void calc_rot(V3 axis, double angle, double* M) {
  const double costh = std::cos(angle), sinth = std::sin(angle);
  const double a[3] = {axis.x, axis.y, axis.z};
  M[0] = costh; M[4] = costh; M[8] = costh;
  M[1] = -axis.z * sinth; M[2] = +axis.y * sinth;
  M[3] = +axis.z * sinth; M[5] = -axis.x * sinth;
  M[6] = -axis.y * sinth; M[7] = +axis.x * sinth;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) M[3 * i + j] = M[3 * i + j] + (1.0 - costh) * a[i] * a[j];
}

V3 rot_apply(const double* M, V3 v) {
  return v3(M[0] * v.x + M[1] * v.y + M[2] * v.z, M[3] * v.x + M[4] * v.y + M[5] * v.z,
            M[6] * v.x + M[7] * v.y + M[8] * v.z);
}

int elem_dim(int t) {
  switch (t) {
    case ELEM_BAR2: return 1;
    case ELEM_TRI3: case ELEM_QUAD4: return 2;
    case ELEM_TETRA4: case ELEM_PYRA5: case ELEM_PENTA6: case ELEM_HEXA8: return 3;
  }
  return 0;
}
int elem_nvtex(int t) {
  switch (t) {
    case ELEM_BAR2: return 2;
    case ELEM_TRI3: return 3;
    case ELEM_QUAD4: return 4;
    case ELEM_TETRA4: return 4;
    case ELEM_PYRA5: return 5;
    case ELEM_PENTA6: return 6;
    case ELEM_HEXA8: return 8;
  }
  return 0;
}

// ---------------------------------------------------------------------------
// XBIN stream reader (native little-endian files only; the endianness word of the
// header is checked).
namespace {
struct XbinIn {
  FILE* f = nullptr;
  bool ok = true;
  template <class T> T get() {
    T v{};
    if (fread(&v, sizeof(T), 1, f) != 1) ok = false;
    return v;
  }
  std::string str(size_t n) {
    std::string s(n, ' ');
    if (n && fread(&s[0], 1, n, f) != n) ok = false;
    return s;
  }
};
std::string rtrim(std::string s) {
  while (!s.empty() && (s.back() == ' ' || s.back() == '\0')) s.pop_back();
  return s;
}
struct XSection {
  int16_t datatype = 0, groupindex = 0, usertype = 0, intsize = 0, realsize = 0;
  std::string name;
  std::vector<int32_t> param;
  std::string string;
  int32_t firstindex = 1, nelem = 0, dim = 0;
};
// xbin_readdatahead (XBIN_DATA.f90:139-186)
bool read_head(XbinIn& in, int version, XSection& s) {
  s.datatype = in.get<int16_t>();
  s.name = rtrim(in.str(32));
  s.groupindex = in.get<int16_t>();
  s.usertype = in.get<int16_t>();
  s.intsize = in.get<int16_t>();
  s.realsize = in.get<int16_t>();
  int16_t nparam = in.get<int16_t>();
  s.param.resize(nparam > 0 ? nparam : 0);
  for (auto& p : s.param) p = in.get<int32_t>();
  if (version >= 2) {
    int16_t strlen_ = in.get<int16_t>();
    s.string = strlen_ > 0 ? in.str(strlen_) : "";
  }
  if (s.datatype == 10 || s.datatype == 20) {
    s.firstindex = in.get<int32_t>();
    s.nelem = in.get<int32_t>();
    s.dim = in.get<int32_t>();
  } else if (s.datatype == 15 || s.datatype == 25) {
    s.nelem = in.get<int32_t>();
    s.dim = in.get<int32_t>();
  }
  return in.ok && s.intsize == 4 && s.realsize == 8;
}
bool read_end(XbinIn& in) { return in.str(3) == "END" && in.ok; }
}  // namespace

bool read_tym(const std::string& path, RawMesh& out, std::string& err) {
  XbinIn in;
  in.f = fopen(path.c_str(), "rb");
  if (!in.f) { err = "cannot open " + path; return false; }
  struct Closer { FILE* f; ~Closer() { fclose(f); } } closer{in.f};
  // xbin_readheader (XBIN_IO.f90:86-106)
  if (in.str(4) != "XBIN") { err = "not a XBIN file"; return false; }
  unsigned char ver[2];
  if (fread(ver, 1, 2, in.f) != 2) { err = "truncated header"; return false; }
  int version = ver[0] * 256 + ver[1];
  unsigned char endian[4];
  if (fread(endian, 1, 4, in.f) != 4) { err = "truncated header"; return false; }
  if (!(endian[0] == 4 && endian[1] == 3 && endian[2] == 2 && endian[3] == 1)) {
    err = "only little-endian XBIN files are supported";
    return false;
  }
  // typhonread_filedef (TYPHON_FMT.f90)
  XSection s;
  if (!read_head(in, version, s) || s.usertype != 1 || !read_end(in)) {
    err = "bad TYPHON file header"; return false;
  }
  int xty_version = s.param.empty() ? 0 : s.param[0];
  // typhonread_umeshheader (TYFMT_MESH.f90)
  XSection mh;
  if (!read_head(in, version, mh) || !read_end(in)) { err = "bad USTMESH header"; return false; }
  int ncellsec, nfacesec, nfacemark;
  if (xty_version == 1) {
    if (mh.param.size() != 7) { err = "bad USTMESH params"; return false; }
    ncellsec = mh.param[4]; nfacesec = mh.param[5]; nfacemark = mh.param[6];
  } else {
    if (mh.param.size() != 8) { err = "bad USTMESH params"; return false; }
    ncellsec = mh.param[4]; nfacesec = mh.param[5]; nfacemark = mh.param[7];
  }
  if (!mh.string.empty()) { err = "shared meshes are not supported"; return false; }
  auto read_elems = [&](int usertype, ElemSection& es) -> bool {
    XSection h;
    if (!read_head(in, version, h) || h.usertype != usertype || h.param.empty()) return false;
    es.type = h.param[0];
    int nelem = h.nelem, nv = h.dim;
    if (nv != elem_nvtex(es.type)) return false;
    es.ielem.resize(nelem);
    if (h.datatype == 15) {  // indexed integer array: index then data
      for (auto& v : es.ielem) v = in.get<int32_t>();
    } else if (h.datatype == 10) {  // ordered: elements numbered from firstindex
      for (int i = 0; i < nelem; ++i) es.ielem[i] = h.firstindex + i;
    } else {
      return false;
    }
    es.vtex.resize((size_t)nelem * nv);
    for (auto& v : es.vtex) v = in.get<int32_t>();
    return read_end(in);
  };
  for (int i = 0; i < ncellsec; ++i) {
    ElemSection es;
    if (!read_elems(12, es)) { err = "bad CELLS section"; return false; }
    out.sections.push_back(std::move(es));
  }
  {  // typhonread_nodes
    XSection h;
    if (!read_head(in, version, h) || h.usertype != 11) { err = "bad NODES section"; return false; }
    out.vtex.resize(h.nelem);
    std::vector<double> buf((size_t)h.nelem * h.dim);
    for (auto& v : buf) v = in.get<double>();
    for (int i = 0; i < h.nelem; ++i)
      out.vtex[i] = v3(buf[(size_t)i * h.dim], buf[(size_t)i * h.dim + 1], buf[(size_t)i * h.dim + 2]);
    if (!read_end(in)) { err = "bad NODES end"; return false; }
  }
  for (int i = 0; i < nfacesec; ++i) {
    ElemSection es;
    if (!read_elems(15, es)) { err = "bad FACES section"; return false; }
    out.sections.push_back(std::move(es));
  }
  for (int i = 0; i < nfacemark; ++i) {  // typhonread_bcmark
    XSection h;
    if (!read_head(in, version, h) || h.usertype != 20) { err = "bad MARK section"; return false; }
    Mark mk;
    mk.family = h.name;
    mk.tags.resize(h.nelem);
    for (auto& v : mk.tags) v = in.get<int32_t>();
    if (!read_end(in)) { err = "bad MARK end"; return false; }
    out.marks.push_back(std::move(mk));
  }
  if (!in.ok) { err = "truncated file"; return false; }
  return true;
}

// ---------------------------------------------------------------------------
namespace {

std::string upper(std::string s) {
  for (auto& c : s) c = (char)toupper((unsigned char)c);
  return s;
}

struct FaceBuilder {
  std::vector<std::vector<int>> facevtex;     // 1-based vertex numbers
  std::vector<int> fc1, fc2;                  // 1-based cell numbers, 0 = none
  std::vector<std::vector<int>> vtexface;     // vertex -> faces (0-based), insertion order

  // same_face (MESHCONNECT.f90:260-283): every vertex of face1 found in face2(1:nsom)
  static bool same_face(const std::vector<int>& f1, const std::vector<int>& f2) {
    size_t n = f1.size();
    if (f2.size() < n) return false;
    bool same = false;
    for (size_t i = 0; i < n; ++i) {
      same = false;
      for (size_t j = 0; j < n; ++j)
        if (f1[i] == f2[j]) { same = true; break; }
      if (!same) break;
    }
    return same;
  }
  // scanface_vtexface (MESHCONNECT.f90:197-225)
  int scan(const std::vector<int>& face) const {
    int is = face[0] - 1;
    for (int f : vtexface[is])
      if (same_face(face, facevtex[f])) return f;
    return -1;
  }
  // ust_create_face (MESHCONNECT.f90:150-195)
  bool create(int icell, const std::vector<int>& face) {
    int iface = scan(face);
    if (iface < 0) {
      int newf = (int)facevtex.size();
      facevtex.push_back(face);
      fc1.push_back(icell);
      fc2.push_back(0);
      for (int v : face) vtexface[v - 1].push_back(newf);
    } else {
      if (fc2[iface] != 0) return false;  // 3 cells on one face
      fc2[iface] = icell;
    }
    return true;
  }
};

}  // namespace

bool build_umesh(const RawMesh& raw, int geo_dim, const std::vector<BcDef>& bcs, UMesh& m,
                 std::string& err) {
  m = UMesh();
  m.dim = geo_dim;
  const int nvtex = (int)raw.vtex.size();
  int maxdim = 0;
  for (auto& s : raw.sections) maxdim = std::max(maxdim, elem_dim(s.type));
  int ncell_int = 0;
  for (auto& s : raw.sections)
    if (elem_dim(s.type) == maxdim) ncell_int += s.nelem();
  m.ncell_int = ncell_int;

  // ---- create_facevtex (create_facevtex.f90:15-220) ----
  FaceBuilder fb;
  fb.vtexface.resize(nvtex);
  for (auto& s : raw.sections) {
    if (elem_dim(s.type) != maxdim) continue;
    const int nv = s.nv();
    for (int ic = 0; ic < s.nelem(); ++ic) {
      int icell = s.ielem[ic];
      const int* e = &s.vtex[(size_t)ic * nv];
      auto mk = [&](std::initializer_list<int> idx) {
        std::vector<int> f;
        for (int k : idx) f.push_back(e[k - 1]);
        return fb.create(icell, f);
      };
      bool ok = true;
      switch (s.type) {
        case ELEM_TRI3:
          ok = mk({1, 2}) && mk({2, 3}) && mk({3, 1});
          break;
        case ELEM_QUAD4:
          ok = mk({1, 2}) && mk({2, 3}) && mk({3, 4}) && mk({4, 1});
          break;
        case ELEM_TETRA4:
          ok = mk({1, 3, 2}) && mk({1, 2, 4}) && mk({2, 3, 4}) && mk({3, 1, 4});
          break;
        case ELEM_PENTA6:
          ok = mk({1, 2, 3}) && mk({4, 5, 6}) && mk({1, 3, 6, 4}) && mk({1, 2, 5, 4}) &&
               mk({2, 3, 6, 5});
          break;
        case ELEM_HEXA8:
          ok = mk({1, 2, 3, 4}) && mk({1, 2, 6, 5}) && mk({5, 6, 7, 8}) && mk({4, 3, 7, 8}) &&
               mk({1, 4, 8, 5}) && mk({2, 3, 7, 6});
          break;
        default:
          err = "unsupported element type";
          return false;
      }
      if (!ok) { err = "bad connectivity: 3 cells found for one face"; return false; }
    }
  }
  const int nface = (int)fb.facevtex.size();

  // ---- reorder_ustconnect (MESHCONNECT.f90:511-606): interior first, boundary reversed ----
  std::vector<int> newidx(nface);
  int nfi = 0, nfl = 0;
  for (int f = 0; f < nface; ++f) {
    if (fb.fc2[f] == 0) { ++nfl; newidx[f] = nface - nfl; }
    else newidx[f] = nfi++;
  }
  m.nface = nface; m.nface_int = nfi; m.nface_lim = nfl;
  m.facevtex.assign(nface, {});
  std::vector<int> c1(nface), c2(nface);
  for (int f = 0; f < nface; ++f) {
    m.facevtex[newidx[f]] = fb.facevtex[f];
    c1[newidx[f]] = fb.fc1[f];
    c2[newidx[f]] = fb.fc2[f];
  }
  for (auto& lst : fb.vtexface)
    for (auto& f : lst) f = newidx[f];
  fb.facevtex = m.facevtex;

  // ---- create_ustboco / seek_bcface_face ----
  for (auto& mk : raw.marks) {
    Boco b;
    b.family = upper(mk.family);
    if (mk.vertex) {  // seek_bcface_vtex.f90:38-45 with face_invtexlist (MESHCONNECT.f90)
      for (int f = nfi; f < nface; ++f) {
        bool same = false;
        for (int v : m.facevtex[f]) {
          same = false;
          for (int t : mk.tags)
            if (v == t || v == 0) { same = true; break; }
          if (!same) break;
        }
        if (same) b.iface.push_back(f);
      }
      if (!b.iface.empty()) m.bocos.push_back(std::move(b));
      continue;
    }
    for (int tag : mk.tags) {
      const std::vector<int>* found = nullptr;
      std::vector<int> face;
      for (auto& s : raw.sections) {
        if (elem_dim(s.type) != maxdim - 1) continue;
        for (int ie = 0; ie < s.nelem(); ++ie)
          if (s.ielem[ie] == tag) {
            face.assign(&s.vtex[(size_t)ie * s.nv()], &s.vtex[(size_t)ie * s.nv()] + s.nv());
            found = &face;
            break;
          }
        if (found) break;
      }
      if (!found) continue;
      int iface = fb.scan(face);
      if (iface >= nfi) b.iface.push_back(iface);
    }
    if (!b.iface.empty()) m.bocos.push_back(std::move(b));
  }
  {
    int nf = 0;
    for (auto& b : m.bocos) nf += (int)b.iface.size();
    if (nf != nfl) { err = "tagged faces do not match boundary faces"; return false; }
  }
  m.ncell = ncell_int + nfl;

  // ---- calc_meshgeom (MESHGEOM.f90:421-461) ----
  m.fnormal.resize(nface); m.fcentre.resize(nface); m.fsurf.resize(nface);
  m.ccentre.assign(m.ncell, V3()); m.cvol.assign(m.ncell, 0.0);
  auto VX = [&](int iv) { return raw.vtex[iv - 1]; };
  // calc_ust_face (MESHGEOM.f90:37-103)
  for (int f = 0; f < nface; ++f) {
    const auto& fv = m.facevtex[f];
    int ns = (int)fv.size();
    if (geo_dim == 2) {
      if (ns != 2) { err = "2D mesh expects 2-vertex faces"; return false; }
      V3 norm = cross(v3(0., 0., 1.), VX(fv[1]) - VX(fv[0]));
      double surf = vabs(norm);
      m.fnormal[f] = norm / surf;
      m.fsurf[f] = surf;
      m.fcentre[f] = 0.5 * (VX(fv[0]) + VX(fv[1]));
    } else if (ns == 3) {
      V3 a = VX(fv[0]), b = VX(fv[1]), c = VX(fv[2]);
      V3 norm = 0.5 * cross(b - a, c - a);
      double surf = vabs(norm);
      m.fnormal[f] = norm / surf;
      m.fsurf[f] = surf;
      m.fcentre[f] = (a + b + c) / 3.0;
    } else if (ns == 4) {
      V3 a = VX(fv[0]), b = VX(fv[1]), c = VX(fv[2]), d = VX(fv[3]);
      V3 norm = 0.5 * cross(b - a, c - a);
      double s1 = vabs(norm);
      V3 cg1 = (a + b + c) / 3.0;
      V3 pt = 0.5 * cross(c - a, d - a);
      double s2 = vabs(pt);
      V3 cg2 = (a + c + d) / 3.0;
      norm = norm + pt;
      double surf = vabs(norm);
      m.fnormal[f] = norm / surf;
      m.fsurf[f] = surf;
      m.fcentre[f] = (s1 * cg1 + s2 * cg2) / (s1 + s2);
    } else {
      err = "faces with 3 or 4 vertices expected"; return false;
    }
  }
  // calc_ust_midcell (MESHGEOM.f90:108-145): at this point fc2 of boundary faces is 0
  std::vector<V3> midcell(m.ncell);
  std::vector<int> nbface(ncell_int, 0);
  for (int f = 0; f < nface; ++f) {
    int i1 = c1[f] - 1, i2 = c2[f] - 1;
    midcell[i1] = midcell[i1] + m.fcentre[f];
    nbface[i1]++;
    if (c2[f] > 0 && c2[f] <= ncell_int) {
      midcell[i2] = midcell[i2] + m.fcentre[f];
      nbface[i2]++;
    }
  }
  for (int c = 0; c < ncell_int; ++c) midcell[c] = midcell[c] / (double)nbface[c];
  // calc_ust_elemvol (MESHGEOM.f90:150-215)
  const double kcg = geo_dim == 2 ? 1.0 / 3.0 : 1.0 / 4.0;
  const double kvol = geo_dim == 2 ? 1.0 / 2.0 : 1.0 / 3.0;
  std::vector<V3> cge(2 * (size_t)nface);
  std::vector<double> vole(2 * (size_t)nface, 0.0);
  auto elemvol = [&](V3 vK, int f, V3& cg, double& vol) {
    V3 vKH = m.fcentre[f] - vK;
    double hauteur = std::fabs(dot(vKH, m.fnormal[f]));
    cg = m.fcentre[f] - kcg * vKH;
    vol = kvol * hauteur * m.fsurf[f];
  };
  for (int f = 0; f < nface; ++f) {
    elemvol(midcell[c1[f] - 1], f, cge[2 * f], vole[2 * f]);
    if (c2[f] > 0 && c2[f] <= ncell_int) elemvol(midcell[c2[f] - 1], f, cge[2 * f + 1], vole[2 * f + 1]);
  }
  // calc_ust_cell (MESHGEOM.f90:220-285)
  for (int f = 0; f < nface; ++f) {
    int i1 = c1[f] - 1;
    m.ccentre[i1] = m.ccentre[i1] + vole[2 * f] * cge[2 * f];
    m.cvol[i1] = m.cvol[i1] + vole[2 * f];
    if (c2[f] > 0 && c2[f] <= ncell_int) {
      int i2 = c2[f] - 1;
      m.ccentre[i2] = m.ccentre[i2] + vole[2 * f + 1] * cge[2 * f + 1];
      m.cvol[i2] = m.cvol[i2] + vole[2 * f + 1];
    }
  }
  for (int c = 0; c < ncell_int; ++c) m.ccentre[c] = m.ccentre[c] / m.cvol[c];
  // calc_ust_checkface (MESHGEOM.f90:290-330)
  for (int f = 0; f < nface; ++f)
    if (c2[f] != 0 && c1[f] > c2[f]) std::swap(c1[f], c2[f]);
  for (int f = 0; f < nface; ++f) {
    V3 v12 = c2[f] != 0 ? m.ccentre[c2[f] - 1] - m.ccentre[c1[f] - 1]
                        : m.fcentre[f] - m.ccentre[c1[f] - 1];
    if (dot(v12, m.fnormal[f]) < 0.0) m.fnormal[f] = -m.fnormal[f];
  }

  // ---- coo_colorgroup (COLOR.f90:33-84), boundary faces have no second cell yet ----
  {
    std::vector<std::vector<int>> vcol(m.ncell);
    auto has = [](const std::vector<int>& l, int c) {
      return std::find(l.begin(), l.end(), c) != l.end();
    };
    for (int f = 0; f < nface; ++f) {
      int a = c1[f] - 1;
      int b = (c2[f] == 0 || c2[f] > m.ncell) ? a : c2[f] - 1;
      bool colored = false;
      for (int ic = 0; ic < (int)m.colors.size(); ++ic) {
        if (!has(vcol[a], ic) && !has(vcol[b], ic)) {
          m.colors[ic].push_back(f);
          vcol[a].push_back(ic);
          vcol[b].push_back(ic);
          colored = true;
          break;
        }
      }
      if (!colored) {
        m.colors.emplace_back();
        int ic = (int)m.colors.size() - 1;
        m.colors[ic].push_back(f);
        vcol[a].push_back(ic);
        vcol[b].push_back(ic);
      }
    }
  }

  // ---- init_connect_grid (init_connect_grid.f90:60-246) ----
  int ncell_lim = 0;
  for (auto& b : m.bocos) {
    b.def = -1;
    for (size_t i = 0; i < bcs.size(); ++i)
      if (upper(bcs[i].family) == b.family && bcs[i].kind != BC_PERIODIC) { b.def = (int)i; break; }
    if (b.def >= 0) {
      // init_ustboco_ghostcell (init_ustboco_ghostcell.f90:44-80)
      const BcDef& d = bcs[b.def];
      b.kind = d.kind;
      b.wall_velocity = d.wall_velocity;
      for (int q = 0; q < 6; ++q) b.data[q] = d.data[q];
      for (int f : b.iface) {
        ++ncell_lim;
        int i1 = c1[f] - 1;
        int g = ncell_int + ncell_lim - 1;
        if (c2[f] != 0) { err = "ghost cell already assigned"; return false; }
        c2[f] = g + 1;
        if (ghost_face_kind(d.kind)) {  // init_ustboco_ghostface.f90:46-56
          m.cvol[g] = 0.0;
          m.ccentre[g] = m.fcentre[f];
        } else if (d.kind == BC_SYMMETRY) {
          V3 fn = m.fnormal[f], gc = m.ccentre[i1];
          m.cvol[g] = m.cvol[i1];
          m.ccentre[g] = gc + (2.0 * dot(m.fcentre[f] - gc, fn)) * fn;
        } else {
          m.cvol[g] = m.cvol[i1];
          m.ccentre[g] = 2.0 * m.fcentre[f] - m.ccentre[i1];
        }
      }
      continue;
    }
    for (size_t i = 0; i < bcs.size(); ++i) {
      if (bcs[i].kind != BC_PERIODIC) continue;
      if (upper(bcs[i].family) == b.family) { b.def = (int)i; b.rlink = 1.0; break; }
      if (upper(bcs[i].partner) == b.family) { b.def = (int)i; b.rlink = -1.0; break; }
    }
    if (b.def < 0) { err = "no boundary definition for family " + b.family; return false; }
    b.kind = BC_PERIODIC;
  }
  for (auto& b : m.bocos) {
    if (b.kind != BC_PERIODIC) continue;
    const BcDef& d = bcs[b.def];
    const int nf = (int)b.iface.size();
    std::vector<V3> vv1(nf);
    if (d.rotation) {  // transloc_per: rotate the face centres about the centre by rlink * angle
      double M[9];
      calc_rot(d.rot_axis, b.rlink * d.rot_angle, M);
      for (int i = 0; i < nf; ++i) vv1[i] = rot_apply(M, m.fcentre[b.iface[i]] - d.rot_centre) + d.rot_centre;
      b.rotation = true;
      calc_rot(d.rot_axis, -b.rlink * d.rot_angle, b.rot);
    } else {
      for (int i = 0; i < nf; ++i) vv1[i] = m.fcentre[b.iface[i]] + b.rlink * d.translation;
    }
    const Boco* b2 = nullptr;
    for (auto& o : m.bocos)
      if (o.kind == BC_PERIODIC && o.def == b.def && o.rlink * b.rlink < 0) {
        if (b2) { err = "too many matching families"; return false; }
        b2 = &o;
      }
    if (!b2 || (int)b2->iface.size() != nf) { err = "no matching periodic family"; return false; }
    // matching_index (GRID_CONNECT.f90:120-150)
    std::vector<int> i1(nf);
    for (int a = 0; a < nf; ++a) {
      double mindist = std::numeric_limits<double>::max();
      int imin = -1;
      for (int c = 0; c < nf; ++c) {
        double dist = vabs(vv1[a] - m.fcentre[b2->iface[c]]);
        if (dist < mindist) { mindist = dist; imin = c; }
      }
      i1[a] = imin;
    }
    for (int f : b.iface) {
      ++ncell_lim;
      if (c2[f] != 0) { err = "ghost cell already assigned"; return false; }
      c2[f] = ncell_int + ncell_lim;
    }
    b.partner_face.resize(nf);
    for (int a = 0; a < nf; ++a) b.partner_face[a] = b2->iface[i1[a]];
    for (int a = 0; a < nf; ++a) {
      int f = b.iface[a], fp = b.partner_face[a];
      int g = c2[f] - 1, icper = c1[fp] - 1;
      V3 dfc = m.ccentre[icper] - m.fcentre[fp];  // translation: vector unchanged
      if (b.rotation) dfc = rot_apply(b.rot, dfc);  // transvec_per(-rlink) (init_connect_grid.f90:218-223)
      m.cvol[g] = m.cvol[icper];
      m.ccentre[g] = m.fcentre[f] + dfc;
    }
  }
  m.fc1.resize(nface); m.fc2.resize(nface);
  for (int f = 0; f < nface; ++f) {
    m.fc1[f] = c1[f] - 1;
    m.fc2[f] = c2[f] - 1;
    if (m.fc2[f] < 0) { err = "boundary face without ghost cell"; return false; }
  }
  return true;
}

}  // namespace ory
