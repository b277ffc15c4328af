// Scene-file loader: CS123 XML scene description + OBJ/MTL meshes.
//
// Restates scenefile_compat::ScenefileLoader (src/scene/scenefile_compat/
// scenefile_loader.cpp:23-319) with the CS123 XML grammar its parser accepts
// (src/scene/scenefile_compat/CS123XmlSceneParser.cpp: <cameradata> with
// pos / look | focus / up / heightangle, <object type="tree"> made of
// <transblock>s holding translate / rotate / scale / matrix and one object
// that is a primitive mesh, a subtree or a master reference), the OBJ / MTL
// subset the Cornell scenes use, polygon triangulation by ear clipping as
// tinyobjloader v1.x does it (projected onto the two axes of the first
// non-degenerate corner), the MTL -> BSDF mapping of
// include/scene/tinyobj_material_conversion.h:13-101 and the emissive
// clusters of consecutive same-material emissive faces.
#include "scene.h"

#include <cctype>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <vector>

namespace pg {

namespace {

// ---------------------------------------------------------------------------
// minimal XML: elements with attributes, nesting, comments and <?...?>
struct XmlNode {
  std::string tag;
  std::map<std::string, std::string> attrs;
  std::vector<std::unique_ptr<XmlNode>> children;
  bool has(const char *k) const { return attrs.count(k) != 0; }
  float num(const char *k) const { return std::strtof(attrs.at(k).c_str(), nullptr); }
};

struct XmlReader {
  const std::string &s;
  size_t i = 0;
  std::string err;
  explicit XmlReader(const std::string &text) : s(text) {}

  void skip_ws() {
    while (i < s.size() && std::isspace((unsigned char)s[i])) {
      ++i;
    }
  }
  bool skip_misc() {
    for (;;) {
      skip_ws();
      if (s.compare(i, 4, "<!--") == 0) {
        size_t e = s.find("-->", i);
        if (e == std::string::npos) {
          err = "unterminated comment";
          return false;
        }
        i = e + 3;
      } else if (s.compare(i, 2, "<?") == 0 || s.compare(i, 2, "<!") == 0) {
        size_t e = s.find('>', i);
        if (e == std::string::npos) {
          err = "unterminated declaration";
          return false;
        }
        i = e + 1;
      } else {
        return true;
      }
    }
  }
  std::unique_ptr<XmlNode> element() {
    if (!skip_misc()) {
      return nullptr;
    }
    if (i >= s.size() || s[i] != '<') {
      err = "expected an element";
      return nullptr;
    }
    ++i;
    auto n = std::make_unique<XmlNode>();
    size_t st = i;
    while (i < s.size() && !std::isspace((unsigned char)s[i]) && s[i] != '>' && s[i] != '/') {
      ++i;
    }
    n->tag = s.substr(st, i - st);
    for (;;) {
      skip_ws();
      if (i >= s.size()) {
        err = "unterminated element " + n->tag;
        return nullptr;
      }
      if (s[i] == '/') {
        if (s.compare(i, 2, "/>") != 0) {
          err = "bad element end";
          return nullptr;
        }
        i += 2;
        return n;
      }
      if (s[i] == '>') {
        ++i;
        break;
      }
      size_t ks = i;
      while (i < s.size() && s[i] != '=' && !std::isspace((unsigned char)s[i])) {
        ++i;
      }
      std::string key = s.substr(ks, i - ks);
      skip_ws();
      if (i >= s.size() || s[i] != '=') {
        err = "attribute without value in " + n->tag;
        return nullptr;
      }
      ++i;
      skip_ws();
      if (i >= s.size() || (s[i] != '"' && s[i] != '\'')) {
        err = "unquoted attribute in " + n->tag;
        return nullptr;
      }
      char q = s[i++];
      size_t vs = i;
      while (i < s.size() && s[i] != q) {
        ++i;
      }
      n->attrs[key] = s.substr(vs, i - vs);
      ++i;
    }
    for (;;) {
      if (!skip_misc()) {
        return nullptr;
      }
      if (s.compare(i, 2, "</") == 0) {
        size_t e = s.find('>', i);
        if (e == std::string::npos) {
          err = "unterminated closing tag";
          return nullptr;
        }
        i = e + 1;
        return n;
      }
      if (i < s.size() && s[i] == '<') {
        auto c = element();
        if (!c) {
          return nullptr;
        }
        n->children.push_back(std::move(c));
      } else {
        // text content is ignored
        while (i < s.size() && s[i] != '<') {
          ++i;
        }
      }
    }
  }
};

// row-major 3x4 affine product a * b
affine compose(const affine &a, const affine &b) {
  affine o;
  for (int r = 0; r < 3; ++r) {
    for (int c = 0; c < 4; ++c) {
      double v = (double)a.m[4 * r] * b.m[c] + (double)a.m[4 * r + 1] * b.m[4 + c] +
                 (double)a.m[4 * r + 2] * b.m[8 + c];
      if (c == 3) {
        v += a.m[4 * r + 3];
      }
      o.m[4 * r + c] = (float)v;
    }
  }
  return o;
}

// rotation by an angle (radians) about the given axis, Rodrigues' matrix
affine rotation(float angle, f3 a) {
  double c = std::cos((double)angle), s = std::sin((double)angle), t = 1.0 - c;
  double x = a.x, y = a.y, z = a.z;
  affine o;
  const double m[12] = {t * x * x + c,     t * x * y - s * z, t * x * z + s * y, 0,
                        t * x * y + s * z, t * y * y + c,     t * y * z - s * x, 0,
                        t * x * z - s * y, t * y * z + s * x, t * z * z + c,     0};
  for (int i = 0; i < 12; ++i) {
    o.m[i] = (float)m[i];
  }
  return o;
}

// ---------------------------------------------------------------------------
// OBJ / MTL
struct ObjMaterial {
  std::string name;
  float kd[3] = {0, 0, 0}, ks[3] = {0, 0, 0}, ke[3] = {0, 0, 0};
  float shininess = 1.f, ior = 1.f;
  int illum = 0;
};

struct Corner {
  int v, vn;
};

bool read_file(const std::string &path, std::string &out) {
  std::ifstream f(path, std::ios::binary);
  if (!f) {
    return false;
  }
  std::stringstream ss;
  ss << f.rdbuf();
  out = ss.str();
  return true;
}

std::string dir_of(const std::string &path) {
  size_t p = path.find_last_of('/');
  return p == std::string::npos ? std::string(".") : path.substr(0, p);
}

bool load_mtl(const std::string &path, std::vector<ObjMaterial> &mats,
              std::map<std::string, int> &ids, std::string &err) {
  std::string text;
  if (!read_file(path, text)) {
    err = "cannot open material library " + path;
    return false;
  }
  std::istringstream in(text);
  std::string line;
  ObjMaterial *cur = nullptr;
  while (std::getline(in, line)) {
    size_t h = line.find('#');
    if (h != std::string::npos) {
      line = line.substr(0, h);
    }
    std::istringstream ls(line);
    std::string key;
    if (!(ls >> key)) {
      continue;
    }
    if (key == "newmtl") {
      ObjMaterial m;
      ls >> m.name;
      ids[m.name] = (int)mats.size();
      mats.push_back(m);
      cur = &mats.back();
    } else if (!cur) {
      continue;
    } else if (key == "Kd") {
      ls >> cur->kd[0] >> cur->kd[1] >> cur->kd[2];
    } else if (key == "Ks") {
      ls >> cur->ks[0] >> cur->ks[1] >> cur->ks[2];
    } else if (key == "Ke") {
      ls >> cur->ke[0] >> cur->ke[1] >> cur->ke[2];
    } else if (key == "Ns") {
      ls >> cur->shininess;
    } else if (key == "Ni") {
      ls >> cur->ior;
    } else if (key == "illum") {
      ls >> cur->illum;
    }
  }
  return true;
}

// tinyobj_material_conversion (include/scene/tinyobj_material_conversion.h)
bool convert_material(const ObjMaterial &m, path_material &o, std::string &err) {
  std::memset(&o, 0, sizeof(o));
  for (int i = 0; i < 3; ++i) {
    o.emission[i] = m.ke[i];
  }
  if (m.illum != 2 && m.illum != 5) {
    err = "material " + m.name + ": unhandled illum " + std::to_string(m.illum) +
          " (only 2 and 5)";
    return false;
  }
  const float eps = 1e-8f;
  float d2 = (m.kd[0] * m.kd[0] + m.kd[1] * m.kd[1]) + m.kd[2] * m.kd[2];
  float s2 = (m.ks[0] * m.ks[0] + m.ks[1] * m.ks[1]) + m.ks[2] * m.ks[2];
  bool diffuse = d2 > eps, specular = s2 > eps;
  const float shininess_threshold = 100;
  if (m.illum == 5) {
    o.type = PATH_BSDF_DIELECTRIC_REFRACTIVE;
    o.specular[0] = o.specular[1] = o.specular[2] = 1.f;
    o.ior = m.ior;
    return true;
  }
  if (diffuse && specular) {
    float td = (m.kd[0] + m.kd[1]) + m.kd[2];
    float ts = (m.ks[0] + m.ks[1]) + m.ks[2];
    float wd = td / (td + ts);
    float wg = (float)(1. - (double)wd);
    for (int i = 0; i < 3; ++i) {
      if (m.kd[i] + m.ks[i] >= 1.f + 1e-4f) {
        err = "material " + m.name + ": diffuse + specular above 1";
        return false;
      }
      o.diffuse[i] = m.kd[i] / wd;
      o.specular[i] = m.ks[i] / wg;
    }
    o.diffuse_weight = wd;
    o.glossy_weight = wg;
    o.shininess = m.shininess;
    o.type = m.shininess > shininess_threshold ? PATH_BSDF_DIFFUSE_MIRROR : PATH_BSDF_DIFFUSE_GLOSSY;
    return true;
  }
  if (diffuse) {
    o.type = PATH_BSDF_DIFFUSE;
    for (int i = 0; i < 3; ++i) {
      o.diffuse[i] = m.kd[i];
    }
    return true;
  }
  if (m.shininess > shininess_threshold) {
    if (!specular) {
      err = "material " + m.name + ": mirror without specular colour";
      return false;
    }
    o.type = PATH_BSDF_MIRROR;
    for (int i = 0; i < 3; ++i) {
      o.specular[i] = m.ks[i];
    }
    return true;
  }
  if (specular) {
    o.type = PATH_BSDF_GLOSSY;
    for (int i = 0; i < 3; ++i) {
      o.specular[i] = m.ks[i];
    }
    o.shininess = m.shininess;
    return true;
  }
  err = "material " + m.name + ": unhandled material settings";
  return false;
}

// point in polygon by ray crossings (W. R. Franklin's pnpoly)
bool pnpoly(const float *vx, const float *vy, float tx, float ty) {
  bool c = false;
  for (int i = 0, j = 2; i < 3; j = i++) {
    if (((vy[i] > ty) != (vy[j] > ty)) &&
        (tx < (vx[j] - vx[i]) * (ty - vy[i]) / (vy[j] - vy[i]) + vx[i])) {
      c = !c;
    }
  }
  return c;
}

// ear clipping of one polygon (tinyobjloader v1.x triangulation)
//
// The steps below follow tinyobjloader v1.1.0's triangulation (projection
// axes, corner epsilon, round limit) so that polygon faces split into the
// same triangles, in the same order, as the reference's loader.  That
// algorithm is used under tinyobjloader's licence:
//
//   The MIT License (MIT)
//   Copyright (c) 2012-2017 Syoyo Fujita and many contributors.
//
//   Permission is hereby granted, free of charge, to any person obtaining a
//   copy of this software and associated documentation files (the
//   "Software"), to deal in the Software without restriction, including
//   without limitation the rights to use, copy, modify, merge, publish,
//   distribute, sublicense, and/or sell copies of the Software, and to
//   permit persons to whom the Software is furnished to do so, subject to
//   the following conditions:
//
//   The above copyright notice and this permission notice shall be included
//   in all copies or substantial portions of the Software.
//
//   THE SOFTWARE IS PROVIDED "AS IS", WITHOUT WARRANTY OF ANY KIND, EXPRESS
//   OR IMPLIED, INCLUDING BUT NOT LIMITED TO THE WARRANTIES OF
//   MERCHANTABILITY, FITNESS FOR A PARTICULAR PURPOSE AND NONINFRINGEMENT.
//   IN NO EVENT SHALL THE AUTHORS OR COPYRIGHT HOLDERS BE LIABLE FOR ANY
//   CLAIM, DAMAGES OR OTHER LIABILITY, WHETHER IN AN ACTION OF CONTRACT,
//   TORT OR OTHERWISE, ARISING FROM, OUT OF OR IN CONNECTION WITH THE
//   SOFTWARE OR THE USE OR OTHER DEALINGS IN THE SOFTWARE.
void triangulate(const std::vector<Corner> &face, const std::vector<float> &v,
                 std::vector<Corner> &out) {
  size_t n = face.size();
  if (n == 3) {
    out.insert(out.end(), face.begin(), face.end());
    return;
  }
  size_t axes[2] = {1, 2};
  for (size_t k = 0; k < n; ++k) {
    const float *a = &v[3 * face[k % n].v], *b = &v[3 * face[(k + 1) % n].v],
                *c = &v[3 * face[(k + 2) % n].v];
    float e0x = b[0] - a[0], e0y = b[1] - a[1], e0z = b[2] - a[2];
    float e1x = c[0] - b[0], e1y = c[1] - b[1], e1z = c[2] - b[2];
    float cx = std::fabs(e0y * e1z - e0z * e1y);
    float cy = std::fabs(e0z * e1x - e0x * e1z);
    float cz = std::fabs(e0x * e1y - e0y * e1x);
    const float eps = 0.0001f;
    if (cx > eps || cy > eps || cz > eps) {
      if (!(cx > cy && cx > cz)) {
        axes[0] = 0;
        if (cz > cx && cz > cy) {
          axes[1] = 1;
        }
      }
      break;
    }
  }
  float area = 0;
  for (size_t k = 0; k < n; ++k) {
    const float *a = &v[3 * face[k].v], *b = &v[3 * face[(k + 1) % n].v];
    area += (a[axes[0]] * b[axes[1]] - a[axes[1]] * b[axes[0]]) * 0.5f;
  }
  std::vector<Corner> rem = face;
  size_t guess = 0;
  int rounds = 10;
  while (rem.size() > 3 && rounds > 0) {
    n = rem.size();
    if (guess >= n) {
      rounds -= 1;
      guess -= n;
    }
    Corner ind[3];
    float vx[3], vy[3];
    for (size_t k = 0; k < 3; ++k) {
      ind[k] = rem[(guess + k) % n];
      vx[k] = v[3 * ind[k].v + axes[0]];
      vy[k] = v[3 * ind[k].v + axes[1]];
    }
    float cross = (vx[1] - vx[0]) * (vy[2] - vy[1]) - (vy[1] - vy[0]) * (vx[2] - vx[1]);
    if (cross * area < 0.0f) {
      guess += 1;
      continue;
    }
    bool overlap = false;
    for (size_t o = 3; o < n; ++o) {
      int vi = rem[(guess + o) % n].v;
      if (pnpoly(vx, vy, v[3 * vi + axes[0]], v[3 * vi + axes[1]])) {
        overlap = true;
        break;
      }
    }
    if (overlap) {
      guess += 1;
      continue;
    }
    out.push_back(ind[0]);
    out.push_back(ind[1]);
    out.push_back(ind[2]);
    size_t removed = (guess + 1) % n;
    while (removed + 1 < n) {
      rem[removed] = rem[removed + 1];
      removed += 1;
    }
    rem.pop_back();
  }
  if (rem.size() == 3) {
    out.insert(out.end(), rem.begin(), rem.end());
  }
}

struct Loader {
  Scene &scene;
  std::map<std::string, uint32_t> loaded; // absolute path -> mesh index
  std::string err;
  explicit Loader(Scene &s) : scene(s) {}

  // load_mesh (scenefile_loader.cpp:120-314)
  bool load_mesh(const std::string &path, const affine &xf) {
    auto it = loaded.find(path);
    if (it != loaded.end()) {
      scene.instances.push_back(xf);
      scene.instance_mesh.push_back(it->second);
      return true;
    }
    std::string text;
    if (!read_file(path, text)) {
      err = "cannot open mesh " + path;
      return false;
    }
    std::vector<float> v, vn;
    std::vector<ObjMaterial> omats;
    std::map<std::string, int> ids;
    int cur_mat = -1;
    struct Tri {
      Corner c[3];
      int mat;
    };
    std::vector<Tri> tris;
    std::istringstream in(text);
    std::string line;
    while (std::getline(in, line)) {
      size_t h = line.find('#');
      if (h != std::string::npos) {
        line = line.substr(0, h);
      }
      std::istringstream ls(line);
      std::string key;
      if (!(ls >> key)) {
        continue;
      }
      if (key == "v") {
        float x, y, z;
        ls >> x >> y >> z;
        v.push_back(x);
        v.push_back(y);
        v.push_back(z);
      } else if (key == "vn") {
        float x, y, z;
        ls >> x >> y >> z;
        vn.push_back(x);
        vn.push_back(y);
        vn.push_back(z);
      } else if (key == "mtllib") {
        std::string f;
        ls >> f;
        if (!load_mtl(dir_of(path) + "/" + f, omats, ids, err)) {
          return false;
        }
      } else if (key == "usemtl") {
        std::string nm;
        ls >> nm;
        auto m = ids.find(nm);
        cur_mat = m == ids.end() ? -1 : m->second;
      } else if (key == "f") {
        std::vector<Corner> face;
        std::string tok;
        while (ls >> tok) {
          int idx[3] = {0, 0, 0};
          int part = 0;
          size_t s0 = 0;
          for (size_t k = 0; k <= tok.size(); ++k) {
            if (k == tok.size() || tok[k] == '/') {
              if (k > s0) {
                idx[part] = std::atoi(tok.substr(s0, k - s0).c_str());
              }
              ++part;
              s0 = k + 1;
              if (part > 2) {
                break;
              }
            }
          }
          int nv = (int)(v.size() / 3), nn = (int)(vn.size() / 3);
          Corner c;
          c.v = idx[0] > 0 ? idx[0] - 1 : nv + idx[0];
          c.vn = idx[2] > 0 ? idx[2] - 1 : (idx[2] < 0 ? nn + idx[2] : -1);
          if (c.v < 0 || c.v >= nv || c.vn >= nn) {
            err = "face index out of range in " + path;
            return false;
          }
          face.push_back(c);
        }
        if (face.size() < 3) {
          continue;
        }
        std::vector<Corner> out;
        triangulate(face, v, out);
        for (size_t k = 0; k + 2 < out.size(); k += 3) {
          tris.push_back({{out[k], out[k + 1], out[k + 2]}, cur_mat});
        }
      }
    }
    uint32_t mat_offset = (uint32_t)scene.materials.size();
    std::vector<bool> emissive;
    for (const ObjMaterial &m : omats) {
      path_material pm;
      if (!convert_material(m, pm, err)) {
        return false;
      }
      emissive.push_back(is_emissive(pm));
      scene.materials.push_back(pm);
    }
    bool in_cluster = false;
    uint32_t cluster_mat = 0, cluster_start = 0;
    for (const Tri &t : tris) {
      if (t.mat < 0) {
        err = "face without material in " + path;
        return false;
      }
      uint32_t mat = (uint32_t)t.mat + mat_offset;
      uint32_t tri_idx = scene.n_tris();
      bool em = emissive[(size_t)t.mat];
      if (em) {
        if (in_cluster && mat != cluster_mat) {
          scene.clusters.insert(scene.clusters.end(), {cluster_mat, cluster_start, tri_idx});
          in_cluster = false;
        }
        if (!in_cluster) {
          in_cluster = true;
          cluster_mat = mat;
          cluster_start = tri_idx;
        }
      } else if (in_cluster) {
        scene.clusters.insert(scene.clusters.end(), {cluster_mat, cluster_start, tri_idx});
        in_cluster = false;
      }
      f3 p[3];
      for (int k = 0; k < 3; ++k) {
        const float *q = &v[3 * t.c[k].v];
        p[k] = mk(q[0], q[1], q[2]);
        scene.tris.insert(scene.tris.end(), {q[0], q[1], q[2]});
      }
      f3 face_n = normalize(cross(p[1] - p[0], p[2] - p[0]));
      for (int k = 0; k < 3; ++k) {
        f3 nn = face_n;
        if (t.c[k].vn >= 0) {
          const float *q = &vn[3 * t.c[k].vn];
          nn = normalize(mk(q[0], q[1], q[2]));
        }
        scene.normals.insert(scene.normals.end(), {nn.x, nn.y, nn.z});
      }
      scene.tri_material.push_back(mat);
    }
    if (in_cluster) {
      scene.clusters.insert(scene.clusters.end(), {cluster_mat, cluster_start, scene.n_tris()});
    }
    uint32_t mesh_idx = (uint32_t)scene.mesh_ends.size();
    scene.mesh_ends.push_back(scene.n_tris());
    scene.cluster_ends_per_mesh.push_back((uint32_t)(scene.clusters.size() / 3));
    scene.instances.push_back(xf);
    scene.instance_mesh.push_back(mesh_idx);
    loaded[path] = mesh_idx;
    return true;
  }

  bool node(const XmlNode &n, const affine &parent, const std::string &dir,
            const std::map<std::string, const XmlNode *> &masters, int depth) {
    if (depth > 64) {
      err = "scene tree too deep (master references form a cycle?)";
      return false;
    }
    affine xf = parent;
    const XmlNode *object = nullptr;
    for (const auto &c : n.children) {
      const XmlNode &e = *c;
      if (e.tag == "translate") {
        affine t = identity_affine();
        t.m[3] = e.num("x");
        t.m[7] = e.num("y");
        t.m[11] = e.num("z");
        xf = compose(xf, t);
      } else if (e.tag == "scale") {
        affine t = identity_affine();
        t.m[0] = e.num("x");
        t.m[5] = e.num("y");
        t.m[10] = e.num("z");
        xf = compose(xf, t);
      } else if (e.tag == "rotate") {
        float ang = (float)(e.num("angle") * M_PI / 180);
        xf = compose(xf, rotation(ang, mk(e.num("x"), e.num("y"), e.num("z"))));
      } else if (e.tag == "matrix") {
        affine t = identity_affine();
        int r = 0;
        for (const auto &row : e.children) {
          if (row->tag != "row" || r >= 4) {
            continue;
          }
          if (r < 3) {
            t.m[4 * r] = row->num("a");
            t.m[4 * r + 1] = row->num("b");
            t.m[4 * r + 2] = row->num("c");
            t.m[4 * r + 3] = row->num("d");
          }
          ++r;
        }
        xf = compose(xf, t);
      } else if (e.tag == "object") {
        object = &e;
      } else if (e.tag == "transblock") {
        if (!node(e, xf, dir, masters, depth + 1)) {
          return false;
        }
      } else {
        err = "unsupported element <" + e.tag + ">";
        return false;
      }
    }
    if (!object) {
      return true;
    }
    auto type = object->attrs.count("type") ? object->attrs.at("type") : std::string();
    if (type == "primitive") {
      std::string name = object->attrs.count("name") ? object->attrs.at("name") : "";
      if (name != "mesh") {
        err = "only mesh primitives are supported, got " + name;
        return false;
      }
      std::string file = object->has("meshfile") ? object->attrs.at("meshfile")
                                                  : (object->has("filename")
                                                         ? object->attrs.at("filename")
                                                         : std::string());
      if (file.empty()) {
        err = "mesh object must specify filename";
        return false;
      }
      return load_mesh(dir + "/" + file, xf);
    }
    if (type == "master") {
      auto m = masters.find(object->attrs.count("name") ? object->attrs.at("name") : "");
      if (m == masters.end()) {
        err = "invalid master object reference";
        return false;
      }
      return tree(*m->second, xf, dir, masters, depth + 1);
    }
    if (type == "tree") {
      return tree(*object, xf, dir, masters, depth + 1);
    }
    err = "invalid object type " + type;
    return false;
  }

  bool tree(const XmlNode &obj, const affine &xf, const std::string &dir,
            const std::map<std::string, const XmlNode *> &masters, int depth) {
    for (const auto &c : obj.children) {
      if (c->tag != "transblock") {
        err = "a tree object holds <transblock> elements only";
        return false;
      }
      if (!node(*c, xf, dir, masters, depth)) {
        return false;
      }
    }
    return true;
  }
};

} // namespace

bool load_scene_xml(const std::string &path, float width_height_ratio, Scene &out,
                    affine &film_to_world, std::string &err) {
  std::string text;
  if (!read_file(path, text)) {
    err = "cannot open scene file " + path;
    return false;
  }
  XmlReader xr(text);
  auto root = xr.element();
  if (!root) {
    err = "XML parse error: " + xr.err;
    return false;
  }
  if (root->tag != "scenefile") {
    err = "missing <scenefile>";
    return false;
  }
  f3 pos = mk(5, 5, 5), up = mk(0, 1, 0), look = mk(-1, -1, -1);
  float height_angle = 45;
  bool focus = false, look_found = false;
  std::map<std::string, const XmlNode *> objects;
  for (const auto &c : root->children) {
    if (c->tag == "cameradata") {
      for (const auto &e : c->children) {
        if (e->tag == "pos") {
          pos = mk(e->num("x"), e->num("y"), e->num("z"));
        } else if (e->tag == "look" || e->tag == "focus") {
          look = mk(e->num("x"), e->num("y"), e->num("z"));
          (e->tag == "focus" ? focus : look_found) = true;
        } else if (e->tag == "up") {
          up = mk(e->num("x"), e->num("y"), e->num("z"));
        } else if (e->tag == "heightangle") {
          height_angle = e->num("v");
        }
      }
    } else if (c->tag == "lightdata") {
      // point / directional lights are rejected (scenefile_loader.cpp:316-319)
      err = "point/directional lights not currently supported";
      return false;
    } else if (c->tag == "object") {
      if (!c->has("name") || c->attrs.at("type") != "tree") {
        err = "top-level <object> elements must be named trees";
        return false;
      }
      objects[c->attrs.at("name")] = c.get();
    } else if (c->tag != "globaldata") {
      err = "unsupported element <" + c->tag + ">";
      return false;
    }
  }
  if (focus && look_found) {
    err = "camera can not have both look and focus";
    return false;
  }
  if (focus) {
    look = look - pos;
  }
  auto r = objects.find("root");
  if (r == objects.end()) {
    err = "scene has no object named root";
    return false;
  }
  Loader loader(out);
  if (!loader.tree(*r->second, identity_affine(), dir_of(path), objects, 0)) {
    err = loader.err;
    return false;
  }
  if (out.mesh_ends.empty()) {
    err = "scene holds no mesh";
    return false;
  }
  ++out.version;
  film_to_world = camera_transform(look, up, pos, height_angle, width_height_ratio);
  return true;
}

} // namespace pg
