// vnf.cpp - .vnf scene files into a context (vmr_load_vnf).
//
// Replaces, for the node types the GPU path renders, what the reference's
// command does between reading a scene and core.Render: nodes.Parse
// (nodes/lex.go, nodes/parser.go: the token rules and the typed field
// syntax), core.AddNode / core.PreRender (core/core.go:29-104: geoms in file
// order, then the geoms lights create in their PreRender, in light order),
// PolyMesh.init (builtin/geom/polymesh/init.go: fan triangulation of
// PolyCount/FaceIdx, per-face ShaderIdx, NormalIdx), the lights' meshes
// (builtin/light/{triangle,disk,sphere,quad}.go createMesh / PreRender) and
// Camera.PreRender (builtin/camera/camera.go:80-98, 109-193).  The result is
// handed to the same C-ABI calls a host binding makes (vmr_mesh_build,
// vmr_sphere_add, vmr_scene_build, vmr_set_shaders, vmr_mesh_set_shading,
// the light setters, vmr_set_camera, vmr_set_pixel_filter).
//
// Numbers follow the reference: a token with '.', 'e' or 'E' is read as a
// float64 and rounded to float32 where the field is float32; integer tokens
// in float fields are converted exactly.  Vector arithmetic for light
// meshes and the camera is float32 without contraction; normalisation is
// a * (1/sqrt((x*x + y*y) + z*z)) (an exact reciprocal square root where the
// reference uses RSQRTSS and one Newton step), the same form the rest of
// libvmr and the project's scene generator use.
//
// Where the reference tolerates an error (prints it and skips the field or
// node), the loader stops with VMR_ERR_INVALID and the file:line in
// vmr_last_error; what the GPU path does not render (textures, the Proc
// handler "wfobj", instances of instances or Procs, lerped motion normals)
// gives VMR_ERR_UNSUPPORTED.  A PolyMesh Transform of one matrix goes to
// vmr_mesh_set_transform, of several keys to vmr_mesh_set_transform_keys;
// GeomInstance to vmr_instance_add; Proc with the "vnf" handler
// (builtin/geom/proc/vnf/vnf.go: the Data file's shaders join the scene's,
// its geoms become the Proc's) to vmr_proc_add; DebugShader to a shader with
// VMR_SH_DEBUG; camera motion keys (LookAt From/To/Roll keys, WorldToLocal
// or LocalToWorld keys) to vmr_set_camera_keys.
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "ctx.h"
#include "vmr.h"

namespace {

// ------------------------------------------------------------------ lexer
enum Tk { kEof, kIdent, kStr, kFloat, kInt, kLBr, kRBr, kLCurl, kRCurl, kComma, kBadNum };

struct Token {
  Tk k = kEof;
  std::string s;
  double f = 0.0;
  int64_t i = 0;
  int line = 0;
};

// nodes/lex.go: identifiers start with a letter or '_' and run to white
// space or one of " [ ] { } , (which is kept); numbers start with '-' or a
// digit and take digits, '-', '.', 'e', 'E'; "#" ends the line; any other
// character is skipped.
class Lexer {
 public:
  explicit Lexer(std::string src) : src_(std::move(src)) {}
  Token next() {
    if (have_peek_) {
      have_peek_ = false;
      return peek_;
    }
    return lex();
  }
  const Token& peek() {
    if (!have_peek_) {
      peek_ = lex();
      have_peek_ = true;
    }
    return peek_;
  }
  int line() const { return line_; }

 private:
  int get() {
    if (pushed_ >= 0) {
      const int c = pushed_;
      pushed_ = -1;
      return c;
    }
    if (pos_ >= src_.size()) return -1;
    const int c = (unsigned char)src_[pos_++];
    if (c == '\n') ++line_;
    if (c == '#') {  // comment: the rest of the line reads as one newline
      while (pos_ < src_.size() && src_[pos_] != '\n') ++pos_;
      if (pos_ < src_.size()) {
        ++pos_;
        ++line_;
      }
      return '\n';
    }
    return c;
  }
  static bool alpha(int c) { return c == '_' || (c >= 'a' && c <= 'z') || (c >= 'A' && c <= 'Z') || c >= 0x80; }

  Token lex() {
    for (;;) {
      const int c = get();
      Token t;
      t.line = line_;
      if (c < 0) return t;
      if (alpha(c)) {
        t.k = kIdent;
        t.s.push_back((char)c);
        for (;;) {
          const int d = get();
          if (d < 0) return Token{kEof, "", 0, 0, line_};
          if (d == '"' || d == '[' || d == ']' || d == '{' || d == '}' || d == ',') {
            pushed_ = d;
            break;
          }
          if (d == ' ' || d == '\t' || d == '\r' || d == '\n') break;
          t.s.push_back((char)d);
        }
        return t;
      }
      if (c == '-' || (c >= '0' && c <= '9')) {
        std::string b(1, (char)c);
        bool is_float = false;
        int d;
        for (;;) {
          d = get();
          if ((d >= '0' && d <= '9') || d == '-') {
            b.push_back((char)d);
          } else if (d == '.' || d == 'e' || d == 'E') {
            is_float = true;
            b.push_back((char)d);
          } else {
            break;
          }
        }
        if (d >= 0) pushed_ = d;
        char* end = nullptr;
        if (is_float) {
          t.f = std::strtod(b.c_str(), &end);
          t.k = (end && *end == 0) ? kFloat : kBadNum;
        } else {
          errno = 0;
          t.i = std::strtoll(b.c_str(), &end, 10);
          t.k = (end && *end == 0 && errno == 0) ? kInt : kBadNum;
        }
        t.s = b;
        return t;
      }
      switch (c) {
        case '[': t.k = kLBr; return t;
        case ']': t.k = kRBr; return t;
        case '{': t.k = kLCurl; return t;
        case '}': t.k = kRCurl; return t;
        case ',': t.k = kComma; return t;
        case '"': {
          t.k = kStr;
          for (;;) {
            const int d = get();
            if (d < 0) return Token{kEof, "", 0, 0, line_};
            if (d == '"') break;
            t.s.push_back((char)d);
          }
          return t;
        }
        default: break;  // white space and unknown characters
      }
    }
  }

  std::string src_;
  size_t pos_ = 0;
  int line_ = 1;
  int pushed_ = -1;
  bool have_peek_ = false;
  Token peek_;
};

// ---------------------------------------------------------- node schemas
enum Ft {
  fInt, fFloat, fBool, fString, fVec3, fMatrix, fPoints, fVec3s, fVec2s, fFloats, fMatrices, fInts, fStrings, fMap
};

struct FieldSpec {
  const char* name;
  Ft t;
  bool required;
};

struct NodeSpec {
  const char* type;
  std::vector<FieldSpec> fields;
};

// The node structs' parseable fields (tag "-" skipped; no ",opt" = required).
const std::vector<NodeSpec>& specs() {
  static const std::vector<NodeSpec> s = {
      {"Globals", {{"XRes", fInt, false}, {"YRes", fInt, false}, {"UseProgress", fBool, false},
                   {"MaxGoRoutines", fInt, false}, {"Camera", fString, false}, {"MaxIter", fInt, false},
                   {"Output", fString, false}}},
      {"Camera", {{"Name", fString, true}, {"Type", fString, true}, {"From", fPoints, true}, {"To", fPoints, true},
                  {"Roll", fFloats, true}, {"Up", fVec3, true}, {"Aspect", fFloat, false}, {"Fov", fFloat, false},
                  {"Focal", fFloat, false}, {"WorldToLocal", fMatrices, false}, {"LocalToWorld", fMatrices, false},
                  {"L", fFloat, false}, {"R", fFloat, false}, {"T", fFloat, false}, {"B", fFloat, false},
                  {"Radius", fFloat, false}}},
      {"PolyMesh", {{"Name", fString, true}, {"RayBias", fFloat, false}, {"Verts", fPoints, true},
                    {"PolyCount", fInts, false}, {"FaceIdx", fInts, false}, {"Shader", fStrings, true},
                    {"ShaderIdx", fInts, false}, {"CalcNormals", fBool, false}, {"IsVisible", fBool, false},
                    {"Transform", fMatrices, false}, {"UV", fVec2s, false}, {"UVIdx", fInts, false},
                    {"Normals", fVec3s, false}, {"NormalIdx", fInts, false}}},
      {"ShaderStd", {{"Name", fString, true}, {"EmissionColour", fMap, false}, {"EmissionStrength", fMap, false},
                     {"Sides", fInt, false}, {"DiffuseColour", fMap, false}, {"DiffuseStrength", fMap, false},
                     {"DiffuseRoughness", fMap, false}, {"Spec1Colour", fMap, false}, {"Spec1Strength", fMap, false},
                     {"Spec1Roughness", fMap, false}, {"Spec1FresnelModel", fString, false},
                     {"Spec1FresnelRefl", fMap, false}, {"Spec1FresnelEdge", fMap, false}, {"IOR", fMap, false}}},
      {"TriLight", {{"Name", fString, true}, {"P0", fVec3, true}, {"P1", fVec3, true}, {"P2", fVec3, true},
                    {"Shader", fString, true}, {"Samples", fInt, true}}},
      {"DiskLight", {{"Name", fString, true}, {"P", fVec3, true}, {"Up", fVec3, true}, {"LookAt", fVec3, true},
                     {"Radius", fFloat, true}, {"Shader", fString, true}, {"Segments", fInt, false},
                     {"Samples", fInt, false}}},
      {"SphereLight", {{"Name", fString, true}, {"P", fVec3, true}, {"Radius", fFloat, true},
                       {"Shader", fString, true}, {"Samples", fInt, false}}},
      {"QuadLight", {{"Name", fString, true}, {"P", fVec3, true}, {"U", fVec3, true}, {"V", fVec3, true},
                     {"Shader", fString, true}, {"Samples", fInt, false}}},
      {"Sphere", {{"Name", fString, true}, {"RayBias", fFloat, false}, {"P", fVec3, true}, {"Radius", fFloat, true},
                  {"Shader", fString, true}}},
      {"GaussianFilter", {{"Name", fString, true}, {"Width", fFloat, true}, {"Res", fInt, true}}},
      {"AiryFilter", {{"Name", fString, true}, {"Width", fFloat, false}, {"Res", fInt, false},
                      {"Peak", fFloat, false}}},
      {"OutputHDR", {{"Filename", fString, true}}},
      {"OutputFloat", {{"Filename", fString, true}}},
      {"DebugShader", {{"Name", fString, true}, {"Sides", fInt, false}, {"Colour", fMap, true}}},
      {"Include", {{"Name", fString, false}, {"Filename", fString, true}}},
      {"GeomInstance", {{"Name", fString, true}, {"Geom", fString, true}, {"BMin", fPoints, true},
                        {"BMax", fPoints, true}, {"Transform", fMatrices, true}}},
      {"Proc", {{"Name", fString, true}, {"Handler", fString, true}, {"Data", fString, true},
                {"BMin", fPoints, true}, {"BMax", fPoints, true}, {"Transform", fMatrices, false}}},
  };
  return s;
}

struct Value {
  Ft t = fInt;
  int64_t i = 0;
  double f = 0.0;
  bool b = false;
  std::string s;
  std::vector<float> v;  // vec3, matrix (column-major), arrays (key-major elements)
  int keys = 0, per = 0;  // arrays: MotionKeys as written, elements per key
  std::vector<int32_t> ints;
  std::vector<std::string> strs;
  float c[3] = {0.f, 0.f, 0.f};  // maps (maps.Constant)
};

struct Node {
  std::string type;
  int line = 0;
  std::map<std::string, Value> f;
  bool has(const char* n) const { return f.count(n) != 0; }
  const Value& at(const char* n) const { return f.at(n); }
};

struct LoadError {
  int code;
  std::string msg;
};

class Parser {
 public:
  Parser(std::string src, std::string name) : lx_(std::move(src)), name_(std::move(name)) {}

  std::vector<Node> parse() {
    std::vector<Node> out;
    for (;;) {
      Token t = lx_.next();
      if (t.k == kEof) break;
      if (t.k != kIdent) fail(t.line, "expected a node name");
      Token b = lx_.next();
      if (b.k != kLCurl) fail(b.line, "expected '{' after node name " + t.s);
      const NodeSpec* spec = nullptr;
      for (const NodeSpec& s : specs())
        if (t.s == s.type) spec = &s;
      if (!spec) fail(t.line, "unknown node type " + t.s);
      out.push_back(node(*spec, t.line));
    }
    return out;
  }

 private:
  [[noreturn]] void fail(int line, const std::string& m) { throw LoadError{VMR_ERR_INVALID, where(line) + m}; }
  std::string where(int line) const { return name_ + ":" + std::to_string(line) + ": "; }

  double number(const char* what) {
    Token t = lx_.next();
    if (t.k == kInt) return (double)t.i;
    if (t.k == kFloat) return t.f;
    fail(t.line, std::string("expected ") + what);
  }
  int64_t integer(const char* what) {
    Token t = lx_.next();
    if (t.k != kInt) fail(t.line, std::string("expected ") + what);
    return t.i;
  }
  void keyword(const char* kw) {
    Token t = lx_.next();
    if (t.k != kIdent || t.s != kw) fail(t.line, std::string("expected type keyword ") + kw);
  }
  // A Matrix4 as written (row after row) stored transposed (Matrix4Transpose).
  void matrix(std::vector<float>& out) {
    float m[16];
    for (int i = 0; i < 16; ++i) m[i] = (float)number("matrix component");
    for (int r = 0; r < 4; ++r)
      for (int c = 0; c < 4; ++c) out.push_back(m[c * 4 + r]);
  }
  // PointArray / Vec3Array / Vec2Array / Float32Array: keys, count, type,
  // then max(keys, 1) * count elements.
  void array(Value& v, const char* kw, int comps) {
    v.keys = (int)integer("number of motion keys");
    v.per = (int)integer("number of elements");
    if (v.keys < 0 || v.per < 0) fail(lx_.line(), "negative array size");
    keyword(kw);
    const int64_t k = v.keys == 0 ? 1 : v.keys;
    const int64_t n = k * (int64_t)v.per * comps;
    if (n > (int64_t)1 << 32) fail(lx_.line(), "array too large");
    v.v.reserve((size_t)n);
    for (int64_t j = 0; j < n; ++j) v.v.push_back((float)number("array element"));
  }

  Value field(Ft t) {
    Value v;
    v.t = t;
    switch (t) {
      case fInt: {
        Token a = lx_.next();
        if (a.k == kFloat) v.i = (int64_t)a.f;
        else if (a.k == kInt) v.i = a.i;
        else fail(a.line, "expected a number");
        break;
      }
      case fFloat: v.f = number("a number"); break;
      case fBool: v.b = integer("0 or 1") != 0; break;
      case fString: {
        Token a = lx_.next();
        if (a.k != kStr) fail(a.line, "expected a string");
        v.s = a.s;
        break;
      }
      case fVec3:
        for (int i = 0; i < 3; ++i) v.v.push_back((float)number("vector component"));
        break;
      case fMatrix:
        keyword("matrix");
        matrix(v.v);
        break;
      case fPoints: array(v, "point", 3); break;
      case fVec3s: array(v, "vec3", 3); break;
      case fVec2s: array(v, "vec2", 2); break;
      case fFloats: array(v, "float", 1); break;
      case fMatrices: {
        v.keys = (int)integer("number of motion keys");
        if (v.keys < 0) fail(lx_.line(), "negative key count");
        keyword("matrix");
        const int k = v.keys == 0 ? 1 : v.keys;
        for (int j = 0; j < k; ++j) matrix(v.v);
        break;
      }
      case fInts: {
        const int64_t n = integer("slice length");
        if (n < 0 || n > ((int64_t)1 << 31)) fail(lx_.line(), "bad slice length");
        keyword("int");
        v.ints.reserve((size_t)n);
        for (int64_t j = 0; j < n; ++j) v.ints.push_back((int32_t)integer("int"));
        break;
      }
      case fStrings: {
        const int64_t n = integer("slice length");
        if (n < 0 || n > ((int64_t)1 << 20)) fail(lx_.line(), "bad slice length");
        keyword("string");
        for (int64_t j = 0; j < n; ++j) {
          Token a = lx_.next();
          if (a.k != kStr) fail(a.line, "expected a string");
          v.strs.push_back(a.s);
        }
        break;
      }
      case fMap: {  // maps.Constant: "rgb r g b" or "float f" (nodes/parser.go rgb, floatmap)
        Token a = lx_.next();
        if (a.k == kIdent && a.s == "rgb") {
          for (int i = 0; i < 3; ++i) v.c[i] = (float)number("RGB component");
        } else if (a.k == kIdent && a.s == "float") {
          const float x = (float)number("float component");
          v.c[0] = v.c[1] = v.c[2] = x;
        } else if (a.k == kIdent && a.s == "rgbtex") {
          throw LoadError{VMR_ERR_UNSUPPORTED, where(a.line) + "texture maps (rgbtex) are not supported"};
        } else {
          fail(a.line, "expected rgb or float");
        }
        break;
      }
    }
    return v;
  }

  Node node(const NodeSpec& spec, int line) {
    Node n;
    n.type = spec.type;
    n.line = line;
    for (;;) {
      Token t = lx_.next();
      if (t.k == kRCurl) break;
      if (t.k != kIdent) fail(t.line, "expected a field name in " + n.type);
      const FieldSpec* fs = nullptr;
      for (const FieldSpec& f : spec.fields)
        if (t.s == f.name) fs = &f;
      if (!fs) fail(t.line, "field \"" + t.s + "\" not found in node " + n.type);
      if (n.f.count(t.s)) fail(t.line, "field " + t.s + " already found in " + n.type);
      n.f[t.s] = field(fs->t);
    }
    for (const FieldSpec& f : spec.fields)
      if (f.required && !n.f.count(f.name))
        fail(line, std::string("required field ") + f.name + " not found in " + n.type);
    return n;
  }

  Lexer lx_;
  std::string name_;
};

// ------------------------------------------------------ float32 helpers
struct F3 {
  float x, y, z;
};
F3 f3(const std::vector<float>& v, size_t o = 0) { return F3{v[o], v[o + 1], v[o + 2]}; }
F3 sub(F3 a, F3 b) { return F3{a.x - b.x, a.y - b.y, a.z - b.z}; }
F3 add(F3 a, F3 b) { return F3{a.x + b.x, a.y + b.y, a.z + b.z}; }
F3 scl(float s, F3 a) { return F3{s * a.x, s * a.y, s * a.z}; }
F3 cross(F3 a, F3 b) { return F3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
F3 nrm(F3 a) {
  float s = a.x * a.x + a.y * a.y;
  s = s + a.z * a.z;
  const float r = 1.0f / std::sqrt(s);
  return F3{a.x * r, a.y * r, a.z * r};
}

// A mesh as the loader hands it to vmr_mesh_build / vmr_mesh_set_shading.
struct MeshOut {
  std::vector<float> verts;  // key-major
  uint32_t n_verts = 0, keys = 1;
  std::vector<uint32_t> idxp;
  std::vector<uint8_t> sidx;
  std::vector<float> normals;  // per vertex (key 0), or empty
  // a motion mesh's Normals with as many keys as its vertices (key-major,
  // mnormals_per_key a key), or empty
  std::vector<float> mnormals;
  uint32_t mnormals_per_key = 0;
  std::vector<uint32_t> shaders;
  float ray_bias = 0.0f;
  bool sphere = false;
  float centre[3] = {0, 0, 0}, radius = 0.f;
  bool has_xf = false;  // PolyMesh.Transform with one non-identity matrix (column-major)
  float xf[16] = {};
  std::vector<float> xkeys;  // PolyMesh.Transform of two or more keys (16 floats each)
  std::string name;
  // 1 GeomInstance (ref: the geom's name), 2 Proc (children: indices into
  // Scene::proc_children); keys: the transform keys; bmin/bmax: key 0's box
  int group = 0;
  std::string ref;
  std::vector<size_t> children;
  std::vector<float> gkeys;
  float bmin[3] = {0, 0, 0}, bmax[3] = {0, 0, 0};
};

struct Scene {
  std::vector<vmr_shader_std> shaders;
  std::map<std::string, uint32_t> shader_id;
  std::vector<MeshOut> geoms;
  std::vector<vmr_tri_light> tris;
  std::vector<vmr_disk_light> disks;
  std::vector<vmr_sphere_light> spheres;
  std::vector<vmr_quad_light> quads;
  std::vector<MeshOut> proc_children;  // geoms reached only through their Proc
  vmr_camera cam{};
  std::vector<float> cam_keys;  // LocalToWorld keys (16 floats each), two or more
  bool has_filter = false;
  vmr_pixel_filter filter{};
  vmr_vnf_info info{};
};

void copy_name(char* dst, size_t cap, const std::string& s) {
  const size_t n = s.size() < cap - 1 ? s.size() : cap - 1;
  std::memcpy(dst, s.data(), n);
  dst[n] = 0;
}

uint32_t shader_of(const Scene& sc, const Node& n, const std::string& name, const std::string& file) {
  auto it = sc.shader_id.find(name);
  if (it == sc.shader_id.end())
    throw LoadError{VMR_ERR_INVALID, file + ":" + std::to_string(n.line) + ": unable to find shader " + name};
  return it->second;
}

// ShaderStd: each field present sets its flag (the reference tests for nil).
vmr_shader_std shader_std(const Node& n) {
  vmr_shader_std s{};
  auto col = [&](const char* f, uint32_t bit, float* dst) {
    if (!n.has(f)) return;
    s.flags |= bit;
    for (int k = 0; k < 3; ++k) dst[k] = n.at(f).c[k];
  };
  auto flt = [&](const char* f, uint32_t bit, float* dst) {
    if (!n.has(f)) return;
    s.flags |= bit;
    *dst = n.at(f).c[0];  // maps.Constant.Float32 reads channel 0
  };
  col("EmissionColour", VMR_SH_EMISSION_COLOUR, s.emission_colour);
  flt("EmissionStrength", VMR_SH_EMISSION_STRENGTH, &s.emission_strength);
  col("DiffuseColour", VMR_SH_DIFFUSE_COLOUR, s.diffuse_colour);
  flt("DiffuseStrength", VMR_SH_DIFFUSE_STRENGTH, &s.diffuse_strength);
  flt("DiffuseRoughness", VMR_SH_DIFFUSE_ROUGHNESS, &s.diffuse_roughness);
  col("Spec1Colour", VMR_SH_SPEC1_COLOUR, s.spec1_colour);
  flt("Spec1Strength", VMR_SH_SPEC1_STRENGTH, &s.spec1_strength);
  flt("Spec1Roughness", VMR_SH_SPEC1_ROUGHNESS, &s.spec1_roughness);
  col("Spec1FresnelRefl", VMR_SH_FRESNEL_REFL, s.spec1_fresnel_refl);
  col("Spec1FresnelEdge", VMR_SH_FRESNEL_EDGE, s.spec1_fresnel_edge);
  flt("IOR", VMR_SH_IOR, &s.ior);
  s.spec1_fresnel = (n.has("Spec1FresnelModel") && n.at("Spec1FresnelModel").s == "Metal") ? 1 : 0;
  return s;
}

// DebugShader (builtin/shader/debug.go:16-57): its Colour as diffuse_colour.
vmr_shader_std debug_shader(const Node& n) {
  vmr_shader_std s{};
  s.flags = VMR_SH_DEBUG;
  for (int k = 0; k < 3; ++k) s.diffuse_colour[k] = n.at("Colour").c[k];
  return s;
}

bool identity(const float* m) {
  for (int i = 0; i < 16; ++i)
    if (m[i] != ((i % 5 == 0) ? 1.0f : 0.0f)) return false;
  return true;
}

// PolyMesh.init (init.go): fan triangulation, per-face shader index,
// normal indices; normals with their own index are de-indexed (each
// triangle corner its own vertex), which leaves every triangle's vertices,
// and so the accelerator, unchanged.
MeshOut poly_mesh(const Node& n, const Scene& sc, const std::string& file) {
  auto where = [&](const std::string& m) { return file + ":" + std::to_string(n.line) + ": PolyMesh: " + m; };
  MeshOut o;
  const Value& V = n.at("Verts");
  o.keys = V.keys == 0 ? 1 : (uint32_t)V.keys;
  o.n_verts = (uint32_t)V.per;
  o.verts = V.v;
  if (n.has("RayBias")) o.ray_bias = (float)n.at("RayBias").f;
  if (n.has("Transform")) {  // an identity changes nothing (the same ray after Setup)
    const Value& T = n.at("Transform");
    const size_t nk = T.v.size() / 16;
    bool all_identity = true;
    for (size_t k = 0; k < nk; ++k) all_identity = all_identity && identity(T.v.data() + 16 * k);
    if (!all_identity) {
      if (nk == 1) {
        o.has_xf = true;
        std::memcpy(o.xf, T.v.data(), sizeof(o.xf));
      } else {
        o.xkeys.assign(T.v.begin(), T.v.begin() + 16 * nk);
      }
    }
  }
  o.name = n.at("Name").s;
  for (const std::string& s : n.at("Shader").strs) o.shaders.push_back(shader_of(sc, n, s, file));
  const std::vector<int32_t> none;
  const std::vector<int32_t>& fi = n.has("FaceIdx") ? n.at("FaceIdx").ints : none;
  const std::vector<int32_t>& ni = n.has("NormalIdx") ? n.at("NormalIdx").ints : none;
  const std::vector<int32_t>& si = n.has("ShaderIdx") ? n.at("ShaderIdx").ints : none;
  // TraceMotionElems uses the normals only with as many keys as the
  // vertices (trace.go:694-712), otherwise N = Ng; the static path uses key 0
  const int nkeys = n.has("Normals") ? (n.at("Normals").keys == 0 ? 1 : n.at("Normals").keys) : 0;
  if (o.keys > 1 && nkeys == (int)o.keys) {  // read at ElemID*3 + corner of each key, not through NormalIdx
    const Value& N = n.at("Normals");
    if (N.v.size() != (size_t)nkeys * N.per * 3) throw LoadError{VMR_ERR_INVALID, where("Normals keys are not whole")};
    o.mnormals = N.v;
    o.mnormals_per_key = (uint32_t)N.per;
  }
  const bool has_n = n.has("Normals") && !n.at("Normals").v.empty() && o.keys == 1;
  std::vector<uint32_t> nidx;
  auto chk = [&](const std::vector<int32_t>& a, size_t i) -> uint32_t {
    if (i >= a.size()) throw LoadError{VMR_ERR_INVALID, where("index array shorter than the polygons need")};
    return (uint32_t)a[i];
  };
  if (n.has("PolyCount")) {
    uint32_t base = 0;
    const std::vector<int32_t>& pc = n.at("PolyCount").ints;
    for (size_t k = 0; k < pc.size(); ++k) {
      uint32_t i = 0;
      for (int j = 0; j < (int)pc[k] - 2; ++j) {
        ++i;
        const uint32_t c[3] = {base, base + i, base + i + 1};
        for (uint32_t q : c) o.idxp.push_back(chk(fi, q));
        if (has_n)
          for (uint32_t q : c) nidx.push_back(ni.empty() ? chk(fi, q) : chk(ni, q));
        if (!si.empty()) o.sidx.push_back((uint8_t)chk(si, k));
      }
      base += (uint32_t)pc[k];
    }
  } else {
    if (!fi.empty()) {
      for (size_t j = 0; j < fi.size(); ++j) {
        o.idxp.push_back((uint32_t)fi[j]);
        if (has_n) nidx.push_back(ni.empty() ? (uint32_t)fi[j] : chk(ni, j));
      }
    } else {
      for (uint32_t j = 0; j < o.n_verts; ++j) {
        o.idxp.push_back(j);
        if (has_n) nidx.push_back(ni.empty() ? j : chk(ni, j));
      }
    }
    for (int32_t s : si) o.sidx.push_back((uint8_t)s);
  }
  if (o.idxp.size() % 3) throw LoadError{VMR_ERR_INVALID, where("face indices are not whole triangles")};
  for (uint32_t v : o.idxp)
    if (v >= o.n_verts) throw LoadError{VMR_ERR_INVALID, where("face index out of range")};
  if (!o.sidx.empty() && o.sidx.size() != o.idxp.size() / 3)
    throw LoadError{VMR_ERR_INVALID, where("ShaderIdx does not give one shader per face")};
  if (has_n) {
    const Value& N = n.at("Normals");
    const size_t nn = (size_t)N.per;
    for (uint32_t q : nidx)
      if (q >= nn) throw LoadError{VMR_ERR_INVALID, where("normal index out of range")};
    bool same = true;
    for (size_t c = 0; c < nidx.size() && same; ++c) same = nidx[c] == o.idxp[c];
    if (same && nn >= o.n_verts) {
      o.normals.assign(N.v.begin(), N.v.begin() + 3 * (size_t)o.n_verts);
    } else {  // de-index: corner c becomes vertex c
      std::vector<float> nv, nn3;
      for (size_t c = 0; c < o.idxp.size(); ++c) {
        for (int k = 0; k < 3; ++k) nv.push_back(o.verts[3 * (size_t)o.idxp[c] + k]);
        for (int k = 0; k < 3; ++k) nn3.push_back(N.v[3 * (size_t)nidx[c] + k]);
      }
      o.verts = nv;
      o.normals = nn3;
      o.n_verts = (uint32_t)o.idxp.size();
      for (size_t c = 0; c < o.idxp.size(); ++c) o.idxp[c] = (uint32_t)c;
    }
  }
  if ((size_t)o.keys * o.n_verts * 3 != o.verts.size())
    throw LoadError{VMR_ERR_INVALID, where("Verts holds the wrong number of values")};
  return o;
}

MeshOut tri_light_mesh(F3 p0, F3 p1, F3 p2, uint32_t shader) {  // triangle.go:537-565
  MeshOut o;
  const F3 N = nrm(cross(sub(p1, p0), sub(p2, p0)));
  o.verts = {p0.x, p0.y, p0.z, p1.x, p1.y, p1.z, p2.x, p2.y, p2.z};
  o.n_verts = 3;
  o.idxp = {0, 1, 2};
  o.normals = {N.x, N.y, N.z, N.x, N.y, N.z, N.x, N.y, N.z};
  o.shaders = {shader};
  return o;
}

MeshOut disk_light_mesh(F3 P, F3 up, F3 at, float R, int segments, uint32_t shader) {  // disk.go:88-90, 224-258
  MeshOut o;
  const F3 N = nrm(sub(at, P));
  const F3 T = nrm(cross(N, up));
  const F3 B = cross(N, T);
  const float pi = 3.14159265358f;
  const float dv = (2.0f * pi) / (float)segments;
  float ang = 0.0f;
  for (int s = 0; s < segments; ++s) {
    const float a1 = ang + dv;
    const float c0 = (float)std::cos((double)ang), s0 = (float)std::sin((double)ang);
    const float c1 = (float)std::cos((double)a1), s1 = (float)std::sin((double)a1);
    const F3 q0 = add(P, add(scl(R * c0, B), scl(R * s0, T)));
    const F3 q1 = add(P, add(scl(R * c1, B), scl(R * s1, T)));
    for (F3 q : {P, q0, q1}) {
      o.verts.insert(o.verts.end(), {q.x, q.y, q.z});
      o.normals.insert(o.normals.end(), {N.x, N.y, N.z});
    }
    ang = ang + dv;
  }
  o.n_verts = (uint32_t)(o.verts.size() / 3);
  for (uint32_t i = 0; i < o.n_verts; ++i) o.idxp.push_back(i);
  o.shaders = {shader};
  return o;
}

MeshOut quad_light_mesh(F3 P, F3 U, F3 V, uint32_t shader) {  // quad.go:41-66, 174-207
  MeshOut o;
  const F3 c[4] = {P, add(P, U), add(add(P, U), V), add(P, V)};
  const F3 N = nrm(cross(U, V));
  for (const F3& q : c) {
    o.verts.insert(o.verts.end(), {q.x, q.y, q.z});
    o.normals.insert(o.normals.end(), {N.x, N.y, N.z});
  }
  o.n_verts = 4;
  o.idxp = {0, 1, 2, 0, 2, 3};  // PolyCount 4, FaceIdx 0 1 2 3 through init's fan
  o.shaders = {shader};
  return o;
}

// Camera.PreRender (camera.go:80-98): TanThetaFocal, then the LocalToWorld
// keys, calcLookatMatrices (:109-193) or matrixCalc (:207-216); keys holds
// them (16 floats each), c.m key 0.
vmr_camera camera(const Node& n, const vmr_vnf_info& info, const std::string& file, std::vector<float>& keys) {
  auto where = [&](const std::string& m) { return file + ":" + std::to_string(n.line) + ": Camera: " + m; };
  vmr_camera c{};
  const float fov = n.has("Fov") ? (float)n.at("Fov").f : 90.0f;
  const float focal = n.has("Focal") ? (float)n.at("Focal").f : 12.0f;
  float aspect = n.has("Aspect") ? (float)n.at("Aspect").f : 0.0f;
  if (aspect == 0.0f) aspect = (float)info.width / (float)info.height;  // core.FrameAspect
  const float pi = 3.14159265358f;
  const float half = fov / 2.0f;
  c.tan_theta_focal = (float)std::tan((double)(half * pi / 180.0f)) * focal;
  c.aspect = aspect;
  c.focal = focal;
  c.radius = n.has("Radius") ? (float)n.at("Radius").f : 0.0f;
  keys.clear();
  const std::string& type = n.at("Type").s;
  if (type == "LookAt") {
    const Value& from = n.at("From");
    const Value& to = n.at("To");
    const Value& roll = n.at("Roll");
    const int nf = from.keys == 0 ? 1 : from.keys, nt = to.keys == 0 ? 1 : to.keys;
    const int nr = roll.keys == 0 ? 1 : roll.keys;
    if ((int)from.v.size() < 3 * nf || (int)to.v.size() < 3 * nt)
      throw LoadError{VMR_ERR_INVALID, where("From/To hold fewer points than their keys")};
    const F3 Up = f3(n.at("Up").v);
    // The array with more keys is walked; the other is lerped at time i/n
    // (not i/(n-1)); Roll, if given, is lerped at the same time.
    const bool by_target = nt > nf;
    const int n_keys = by_target ? nt : nf;
    auto lerp_key = [](const Value& a, int na, float time) {
      const float k = time * (float)(na - 1);
      const float t = k - std::floor(k);
      const int key = (int)std::floor(k), key2 = (int)std::ceil(k);
      const float* p = a.v.data() + 3 * key;
      const float* q = a.v.data() + 3 * key2;
      return F3{(1.0f - t) * p[0] + t * q[0], (1.0f - t) * p[1] + t * q[1], (1.0f - t) * p[2] + t * q[2]};
    };
    for (int i = 0; i < n_keys; ++i) {
      const float time = (float)i / (float)n_keys;
      const F3 From = by_target ? lerp_key(from, nf, time) : f3(from.v, 3 * (size_t)i);
      const F3 To = by_target ? f3(to.v, 3 * (size_t)i) : lerp_key(to, nt, time);
      const F3 W = nrm(sub(From, To));  // W points away from the target
      const F3 u = nrm(cross(Up, W));
      const F3 v = nrm(cross(u, W));
      float r = 0.0f;
      if (!roll.v.empty()) {
        const float k = time * (float)(nr - 1);
        const float t = k - std::floor(k);
        const int key = (int)std::floor(k), key2 = (int)std::ceil(k);
        r = (1.0f - t) * roll.v[key] + t * roll.v[key2];
      }
      const float cr = (float)std::cos((double)r), sr = (float)std::sin((double)r);
      const F3 U = add(scl(cr, u), scl(sr, v));
      const F3 Vv = add(scl(-sr, u), scl(cr, v));
      // Matrix4Mul(Matrix4Translate(From), Matrix4Basis(U, V, W))
      float tr[16], basis[16], m[16];
      vmr::anim::identity(tr);
      tr[12] = From.x;
      tr[13] = From.y;
      tr[14] = From.z;
      const float bz[16] = {U.x, U.y, U.z, 0.f, Vv.x, Vv.y, Vv.z, 0.f, W.x, W.y, W.z, 0.f, 0.f, 0.f, 0.f, 1.f};
      std::memcpy(basis, bz, sizeof(basis));
      vmr::anim::mul(tr, basis, m);
      keys.insert(keys.end(), m, m + 16);
    }
  } else {
    // matrixCalc: the given LocalToWorld keys, then the inverse of each
    // WorldToLocal key (Matrix4Inverse; its ok flag is ignored)
    if (n.has("LocalToWorld")) {
      const Value& M = n.at("LocalToWorld");
      keys.insert(keys.end(), M.v.begin(), M.v.end());
    }
    if (n.has("WorldToLocal")) {
      const Value& M = n.at("WorldToLocal");
      for (size_t k = 0; k + 16 <= M.v.size(); k += 16) {
        float inv[16];
        vmr::anim::inverse(M.v.data() + k, inv);
        keys.insert(keys.end(), inv, inv + 16);
      }
    }
  }
  if (keys.empty()) {  // no keys: Matrix4Identity (camera.go:223)
    float I[16];
    vmr::anim::identity(I);
    keys.assign(I, I + 16);
  }
  std::memcpy(c.m, keys.data(), sizeof(c.m));
  return c;
}

MeshOut sphere_geom(const Node& n, const Scene& sc, const std::string& file) {
  MeshOut o;
  o.sphere = true;
  o.name = n.at("Name").s;
  for (int k = 0; k < 3; ++k) o.centre[k] = n.at("P").v[k];
  o.radius = (float)n.at("Radius").f;
  o.shaders = {shader_of(sc, n, n.at("Shader").s, file)};
  return o;
}

// A file named by a node: relative to the naming file's directory if it
// exists there, else as given (the reference opens it from the working
// directory).
std::string near(const std::string& from, const std::string& name) {
  const size_t slash = from.find_last_of('/');
  if (slash == std::string::npos || (!name.empty() && name[0] == '/')) return name;
  const std::string rel = from.substr(0, slash + 1) + name;
  std::ifstream probe(rel);
  return probe ? rel : name;
}

std::vector<Node> parse_file(const std::string& path);

// Proc.PreRender with the "vnf" handler (builtin/geom/proc/vnf/vnf.go:18-55):
// the Data file is parsed, its shaders join the scene's (core.AddNode; a
// name already taken keeps its first shader), its geoms (PolyMesh, Sphere)
// become the Proc's children in file order; other nodes are skipped, as the
// handler logs and skips them.  Data is found relative to the scene file's
// directory, then as given.  The "wfobj" handler (Wavefront OBJ) is not
// supported.
void proc_geoms(const Node& n, Scene& sc, const std::string& file, MeshOut& o) {
  auto where = [&](const std::string& m) { return file + ":" + std::to_string(n.line) + ": Proc: " + m; };
  const std::string& handler = n.at("Handler").s;
  if (handler == "wfobj") throw LoadError{VMR_ERR_UNSUPPORTED, where("the wfobj (Wavefront OBJ) handler is not supported")};
  if (handler != "vnf") throw LoadError{VMR_ERR_INVALID, where("unable to find handler " + handler)};
  const std::string data = near(file, n.at("Data").s);
  const std::vector<Node> sub = parse_file(data);
  for (const Node& c : sub)
    if ((c.type == "ShaderStd" || c.type == "DebugShader") && !sc.shader_id.count(c.at("Name").s)) {
      sc.shader_id[c.at("Name").s] = (uint32_t)sc.shaders.size();
      sc.shaders.push_back(c.type == "ShaderStd" ? shader_std(c) : debug_shader(c));
    }
  for (const Node& c : sub) {
    if (c.type == "PolyMesh") {
      o.children.push_back(sc.proc_children.size());
      sc.proc_children.push_back(poly_mesh(c, sc, data));
    } else if (c.type == "Sphere") {
      o.children.push_back(sc.proc_children.size());
      sc.proc_children.push_back(sphere_geom(c, sc, data));
    } else if (c.type == "GeomInstance" || c.type == "Proc") {
      throw LoadError{VMR_ERR_UNSUPPORTED, where("instances and Procs inside a Proc are not supported")};
    }
  }
  if (o.children.empty()) throw LoadError{VMR_ERR_INVALID, where("no geoms in " + data)};
}

bool is_light(const Node& n) {
  return n.type == "TriLight" || n.type == "DiskLight" || n.type == "SphereLight" || n.type == "QuadLight";
}
bool is_geom(const Node& n) {
  return n.type == "PolyMesh" || n.type == "Sphere" || n.type == "GeomInstance" || n.type == "Proc";
}

// A node and the file it came from.
struct Item {
  const Node* n;
  std::string file;
};

// One geom slot of the scene, in core.AddNode / PreRender order: a geom
// node (added when parsed) or a light's own mesh (added by the light's
// PreRender).
struct Slot {
  Item it;
  bool light_mesh;
};

MeshOut geom_of(const Item& it, Scene& sc) {
  const Node& n = *it.n;
  if (n.type == "PolyMesh") return poly_mesh(n, sc, it.file);
  if (n.type == "Sphere") return sphere_geom(n, sc, it.file);
  MeshOut o;  // GeomInstance or Proc
  o.name = n.at("Name").s;
  o.group = n.type == "GeomInstance" ? 1 : 2;
  const Value &lo = n.at("BMin"), &hi = n.at("BMax");
  if (lo.v.size() < 3 || hi.v.size() < 3)
    throw LoadError{VMR_ERR_INVALID, it.file + ":" + std::to_string(n.line) + ": " + n.type + " needs BMin and BMax"};
  for (int k = 0; k < 3; ++k) {
    o.bmin[k] = lo.v[k];
    o.bmax[k] = hi.v[k];
  }
  if (n.has("Transform")) o.gkeys = n.at("Transform").v;
  if (o.group == 1) {
    o.ref = n.at("Geom").s;
    if (o.gkeys.empty())
      throw LoadError{VMR_ERR_INVALID, it.file + ":" + std::to_string(n.line) + ": GeomInstance needs a Transform"};
  } else {
    proc_geoms(n, sc, it.file, o);
  }
  return o;
}

// A light's own mesh (its PreRender) and its table entry pointing at geom.
void light_of(const Item& it, Scene& sc, uint32_t geom) {
  const Node& n = *it.n;
  const std::string& file = it.file;
  const uint32_t sh = shader_of(sc, n, n.at("Shader").s, file);
  const int samples = n.has("Samples") ? (int)n.at("Samples").i : 1;
  if (n.type == "TriLight") {
    const F3 p0 = f3(n.at("P0").v), p1 = f3(n.at("P1").v), p2 = f3(n.at("P2").v);
    sc.geoms[geom] = tri_light_mesh(p0, p1, p2, sh);
    vmr_tri_light l{};
    std::memcpy(l.p0, &p0, 12);
    std::memcpy(l.p1, &p1, 12);
    std::memcpy(l.p2, &p2, 12);
    l.samples = samples;
    l.shader = sh;
    l.geom = geom;
    sc.tris.push_back(l);
  } else if (n.type == "DiskLight") {
    const F3 P = f3(n.at("P").v), up = f3(n.at("Up").v), at = f3(n.at("LookAt").v);
    const float R = (float)n.at("Radius").f;
    const int seg = n.has("Segments") ? (int)n.at("Segments").i : 20;
    if (seg < 1 || seg > 65536) throw LoadError{VMR_ERR_INVALID, file + ": DiskLight Segments out of range"};
    sc.geoms[geom] = disk_light_mesh(P, up, at, R, seg, sh);
    vmr_disk_light l{};
    std::memcpy(l.P, &P, 12);
    std::memcpy(l.up, &up, 12);
    std::memcpy(l.lookat, &at, 12);
    l.radius = R;
    l.samples = samples;
    l.shader = sh;
    l.geom = geom;
    sc.disks.push_back(l);
  } else if (n.type == "SphereLight") {
    MeshOut o;
    o.sphere = true;
    for (int k = 0; k < 3; ++k) o.centre[k] = n.at("P").v[k];
    o.radius = (float)n.at("Radius").f;
    o.shaders = {sh};
    sc.geoms[geom] = o;
    vmr_sphere_light l{};
    std::memcpy(l.P, o.centre, 12);
    l.radius = o.radius;
    l.samples = samples;
    l.shader = sh;
    l.geom = geom;
    sc.spheres.push_back(l);
  } else {
    const F3 P = f3(n.at("P").v), U = f3(n.at("U").v), V = f3(n.at("V").v);
    sc.geoms[geom] = quad_light_mesh(P, U, V, sh);
    vmr_quad_light l{};
    std::memcpy(l.p0, &P, 12);
    std::memcpy(l.e1, &U, 12);
    std::memcpy(l.e2, &V, 12);
    l.shader = sh;
    l.geom = geom;
    sc.quads.push_back(l);
  }
}

// core.AddNode and core.PreRender (core/core.go:29-104) over the file's
// nodes.  Parsing adds every node: geoms join the scene then, in file order.
// PreRender then runs over the nodes round by round: a light creates its
// mesh (a new geom), an Include (builtin/misc/include.go) parses its file,
// whose nodes are added at that point and PreRender'ed in the next round.
// Shaders, Globals, the pixel filter and the camera are looked up over all
// nodes once the rounds are done (a later node of a name wins, as core's
// node map does).
Scene build_scene(const std::vector<Node>& nodes, const std::string& file, int flags,
                  std::vector<std::vector<Node>>& included) {
  Scene sc;
  std::vector<Item> all, round;
  std::vector<Slot> slots;
  std::vector<Item> lights;
  auto add = [&](const Item& it) {
    all.push_back(it);
    if (is_geom(*it.n)) slots.push_back(Slot{it, false});
    round.push_back(it);
  };
  for (const Node& n : nodes) add(Item{&n, file});
  for (int depth = 0; !round.empty(); ++depth) {
    if (depth > 16) throw LoadError{VMR_ERR_INVALID, file + ": Include nesting deeper than 16"};
    std::vector<Item> cur;
    cur.swap(round);
    for (const Item& it : cur) {
      if (is_light(*it.n)) {
        slots.push_back(Slot{it, true});
      } else if (it.n->type == "Include") {
        const std::string path = near(it.file, it.n->at("Filename").s);
        included.push_back(parse_file(path));
        for (const Node& c : included.back()) add(Item{&c, path});
      }
    }
  }
  // core.Init's defaults; a Globals node starts from its own (256 x 256, MaxIter 0)
  sc.info.width = 1024;
  sc.info.height = 1024;
  sc.info.max_iter = 16;
  std::string cam_name = "camera";
  for (const Item& it : all) {
    const Node& n = *it.n;
    if (n.type == "Globals") {
      sc.info.width = n.has("XRes") ? (uint32_t)n.at("XRes").i : 256;
      sc.info.height = n.has("YRes") ? (uint32_t)n.at("YRes").i : 256;
      sc.info.max_iter = n.has("MaxIter") ? (int)n.at("MaxIter").i : 0;
      cam_name = n.has("Camera") && !n.at("Camera").s.empty() ? n.at("Camera").s : "camera";
    } else if (n.type == "ShaderStd" || n.type == "DebugShader") {
      sc.shader_id[n.at("Name").s] = (uint32_t)sc.shaders.size();
      sc.shaders.push_back(n.type == "ShaderStd" ? shader_std(n) : debug_shader(n));
    } else if (n.type == "OutputHDR") {
      copy_name(sc.info.output_hdr, sizeof(sc.info.output_hdr), n.at("Filename").s);
    } else if (n.type == "OutputFloat") {
      copy_name(sc.info.output_float, sizeof(sc.info.output_float), n.at("Filename").s);
    } else if (n.type == "GaussianFilter" || n.type == "AiryFilter") {
      sc.has_filter = true;
      sc.filter = vmr_pixel_filter{n.type == "GaussianFilter" ? VMR_FILTER_GAUSSIAN : VMR_FILTER_AIRY,
                                   n.has("Res") ? (int)n.at("Res").i : 49,
                                   n.has("Width") ? (float)n.at("Width").f : 6.0f,
                                   n.has("Peak") ? (float)n.at("Peak").f : 4.0f};
    }
  }
  if (sc.info.width == 0 || sc.info.height == 0 || sc.info.width > 4096 || sc.info.height > 4096)
    throw LoadError{VMR_ERR_INVALID, file + ": Globals XRes/YRes must be in [1, 4096]"};
  // the scene's geoms in slot order; the light tables in the order the
  // lights were added (parse order, then the included files')
  sc.geoms.resize(slots.size());
  std::vector<uint32_t> light_slot;
  std::vector<Item> light_items;
  for (size_t i = 0; i < slots.size(); ++i)
    if (!slots[i].light_mesh) sc.geoms[i] = geom_of(slots[i].it, sc);
  for (const Item& it : all)
    if (is_light(*it.n))
      for (size_t i = 0; i < slots.size(); ++i)
        if (slots[i].light_mesh && slots[i].it.n == it.n) light_of(it, sc, (uint32_t)i);
  // the render's camera (core/render.go:147-162): the last Camera of the name
  const Item* cam = nullptr;
  for (const Item& it : all)
    if (it.n->type == "Camera" && it.n->at("Name").s == cam_name) cam = &it;
  if (!cam) throw LoadError{VMR_ERR_INVALID, file + ": no camera named " + cam_name};
  sc.cam = camera(*cam->n, sc.info, cam->file, sc.cam_keys);
  copy_name(sc.info.camera, sizeof(sc.info.camera), cam_name);
  (void)flags;
  return sc;
}

std::vector<Node> parse_file(const std::string& path) {
  std::ifstream in(path, std::ios::binary);
  if (!in) throw LoadError{VMR_ERR_INVALID, std::string("cannot open ") + path};
  std::stringstream ss;
  ss << in.rdbuf();
  Parser p(ss.str(), path);
  return p.parse();
}

int fail(vmr_ctx* ctx, int code, const std::string& m) {
  ctx->err = m;
  return code;
}

// One mesh or sphere through the C ABI (vmr_mesh_build or vmr_sphere_add,
// then its transform).
int upload_geom(vmr_ctx* ctx, const MeshOut& g, int mode, uint32_t* id) {
  if (g.sphere) return vmr_sphere_add(ctx, g.centre, g.radius, id);
  vmr_mesh_input mi{};
  mi.verts = g.verts.data();
  mi.n_verts = g.n_verts;
  mi.motion_keys = g.keys;
  mi.idxp = g.idxp.data();
  mi.n_tris = (uint32_t)(g.idxp.size() / 3);
  mi.ray_bias = g.ray_bias;
  mi.motion_mode = mode;
  mi.shader_idx = g.sidx.empty() ? nullptr : g.sidx.data();
  int rc = vmr_mesh_build(ctx, &mi, id);
  if (rc == VMR_OK && g.has_xf) rc = vmr_mesh_set_transform(ctx, *id, g.xf);
  if (rc == VMR_OK && !g.xkeys.empty())
    rc = vmr_mesh_set_transform_keys(ctx, *id, g.xkeys.data(), (uint32_t)(g.xkeys.size() / 16));
  return rc;
}

int set_shading(vmr_ctx* ctx, uint32_t id, const MeshOut& g) {
  int rc = vmr_mesh_set_shading(ctx, id, g.shaders.data(), (uint32_t)g.shaders.size(),
                                g.normals.empty() ? nullptr : g.normals.data());
  if (rc == VMR_OK && !g.mnormals.empty())
    rc = vmr_mesh_set_motion_normals(ctx, id, g.mnormals.data(), g.mnormals_per_key, g.keys);
  return rc;
}

}  // namespace

extern "C" int vmr_get_camera(vmr_ctx* ctx, vmr_camera* camera) {
  if (!ctx || !camera) return VMR_ERR_INVALID;
  if (!ctx->render.has_camera) return fail(ctx, VMR_ERR_INVALID, "no camera set");
  *camera = ctx->render.camera;
  return VMR_OK;
}

extern "C" int vmr_load_vnf(vmr_ctx* ctx, const char* path, int flags, vmr_vnf_info* info) {
  if (!ctx || !path) return VMR_ERR_INVALID;
  Scene sc;
  std::vector<std::vector<Node>> included;  // the Include files' nodes, alive while the scene is built
  try {
    const std::vector<Node> nodes = parse_file(path);
    sc = build_scene(nodes, path, flags, included);
  } catch (const LoadError& e) {
    return fail(ctx, e.code, e.msg);
  } catch (const std::exception& e) {
    return fail(ctx, VMR_ERR_INVALID, std::string(path) + ": " + e.what());
  }
  // upload through the C ABI, as a host binding would: meshes and spheres
  // first, then the instances and Procs that reference them
  const int mode = (flags & VMR_VNF_MOTION_FIXED) ? VMR_MOTION_FIXED : VMR_MOTION_FAITHFUL;
  std::vector<uint32_t> ids(sc.geoms.size()), child_ids(sc.proc_children.size());
  std::map<std::string, size_t> by_name;
  for (size_t i = 0; i < sc.geoms.size(); ++i) {
    const MeshOut& g = sc.geoms[i];
    if (!g.name.empty() && !by_name.count(g.name)) by_name[g.name] = i;
    if (g.group) continue;
    const int rc = upload_geom(ctx, g, mode, &ids[i]);
    if (rc != VMR_OK) return rc;
  }
  for (size_t i = 0; i < sc.proc_children.size(); ++i) {
    const int rc = upload_geom(ctx, sc.proc_children[i], mode, &child_ids[i]);
    if (rc != VMR_OK) return rc;
  }
  for (size_t i = 0; i < sc.geoms.size(); ++i) {
    const MeshOut& g = sc.geoms[i];
    if (!g.group) continue;
    const uint32_t nk = (uint32_t)(g.gkeys.size() / 16);
    int rc;
    if (g.group == 1) {
      auto it = by_name.find(g.ref);
      if (it == by_name.end() || sc.geoms[it->second].group)
        return fail(ctx, it == by_name.end() ? VMR_ERR_INVALID : VMR_ERR_UNSUPPORTED,
                    std::string(path) + ": GeomInstance " + g.name + ": unable to find geom " + g.ref +
                        (it == by_name.end() ? "" : " (instances of instances or Procs are not supported)"));
      rc = vmr_instance_add(ctx, ids[it->second], g.gkeys.data(), nk, g.bmin, g.bmax, &ids[i]);
    } else {
      std::vector<uint32_t> ch;
      for (size_t c : g.children) ch.push_back(child_ids[c]);
      rc = vmr_proc_add(ctx, ch.data(), (uint32_t)ch.size(), nk ? g.gkeys.data() : nullptr, nk, g.bmin, g.bmax,
                        &ids[i]);
    }
    if (rc != VMR_OK) return rc;
  }
  int rc = vmr_scene_build(ctx, ids.data(), (uint32_t)ids.size());
  if (rc == VMR_OK) rc = vmr_set_shaders(ctx, sc.shaders.data(), (uint32_t)sc.shaders.size());
  for (size_t g = 0; g < sc.geoms.size() && rc == VMR_OK; ++g)
    if (!sc.geoms[g].group) rc = set_shading(ctx, ids[g], sc.geoms[g]);
  for (size_t g = 0; g < sc.proc_children.size() && rc == VMR_OK; ++g)
    rc = set_shading(ctx, child_ids[g], sc.proc_children[g]);
  auto remap = [&](uint32_t g) { return ids[g]; };
  for (auto& l : sc.tris) l.geom = remap(l.geom);
  for (auto& l : sc.disks) l.geom = remap(l.geom);
  for (auto& l : sc.spheres) l.geom = remap(l.geom);
  for (auto& l : sc.quads) l.geom = remap(l.geom);
  if (rc == VMR_OK) rc = vmr_set_lights(ctx, sc.tris.data(), (uint32_t)sc.tris.size());
  if (rc == VMR_OK) rc = vmr_set_disk_lights(ctx, sc.disks.data(), (uint32_t)sc.disks.size());
  if (rc == VMR_OK) rc = vmr_set_sphere_lights(ctx, sc.spheres.data(), (uint32_t)sc.spheres.size());
  if (rc == VMR_OK) rc = vmr_set_quad_lights(ctx, sc.quads.data(), (uint32_t)sc.quads.size());
  const float black[3] = {0.f, 0.f, 0.f};
  if (rc == VMR_OK) rc = vmr_set_env_light(ctx, black);
  if (rc == VMR_OK) rc = vmr_set_camera(ctx, &sc.cam);
  if (rc == VMR_OK && sc.cam_keys.size() > 16)
    rc = vmr_set_camera_keys(ctx, sc.cam_keys.data(), (uint32_t)(sc.cam_keys.size() / 16));
  if (rc == VMR_OK) {
    vmr_pixel_filter none{VMR_FILTER_BOX, 0, 0.f, 0.f};
    rc = vmr_set_pixel_filter(ctx, sc.has_filter ? &sc.filter : &none);
  }
  if (rc != VMR_OK) return rc;
  sc.info.n_geoms = (uint32_t)ids.size();
  sc.info.n_shaders = (uint32_t)sc.shaders.size();
  sc.info.n_lights = (uint32_t)(sc.tris.size() + sc.disks.size() + sc.spheres.size() + sc.quads.size());
  if (info) *info = sc.info;
  return VMR_OK;
}
