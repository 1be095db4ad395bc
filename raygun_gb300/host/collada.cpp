// collada.cpp -- Collada (.dae) and .rgmat.json ingest of the C++ facade (include/rg/collada.hpp).
//
// A small XML reader (elements, attributes, text; comments, processing instructions and DOCTYPE
// skipped; the five predefined entities decoded) and a small JSON reader are enough for the files
// Raygun ships: Blender's Collada 1.4.1 export and the resource manager's material files.
#include "../../include/rg/collada.hpp"

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <functional>
#include <map>
#include <sstream>

namespace rg {

namespace {

// ---- XML ---------------------------------------------------------------------------------------
struct XmlNode {
    std::string tag;
    std::vector<std::pair<std::string, std::string>> attrs;
    std::string text;
    std::vector<std::unique_ptr<XmlNode>> kids;

    const std::string* attr(const char* name) const {
        for (const auto& a : attrs)
            if (a.first == name) return &a.second;
        return nullptr;
    }
    std::string attrOr(const char* name, const std::string& dflt) const {
        const std::string* a = attr(name);
        return a ? *a : dflt;
    }
    const XmlNode* child(const char* name) const {
        for (const auto& k : kids)
            if (k->tag == name) return k.get();
        return nullptr;
    }
    std::vector<const XmlNode*> children(const char* name) const {
        std::vector<const XmlNode*> out;
        for (const auto& k : kids)
            if (k->tag == name) out.push_back(k.get());
        return out;
    }
};

class XmlReader {
  public:
    explicit XmlReader(const std::string& s) : s_(s) {}

    std::unique_ptr<XmlNode> document() {
        skipMisc();
        if (pos_ >= s_.size() || s_[pos_] != '<') fail("no root element");
        auto root = element();
        return root;
    }

  private:
    [[noreturn]] void fail(const std::string& what) const {
        throw ColladaError("XML: " + what + " at byte " + std::to_string(pos_));
    }
    bool startsWith(const char* p) const { return s_.compare(pos_, std::strlen(p), p) == 0; }
    void skipWs() {
        while (pos_ < s_.size() && std::isspace((unsigned char)s_[pos_])) ++pos_;
    }
    void skipPast(const char* end) {
        size_t e = s_.find(end, pos_);
        if (e == std::string::npos) fail(std::string("unterminated construct, expected ") + end);
        pos_ = e + std::strlen(end);
    }
    // whitespace, comments, processing instructions, DOCTYPE
    void skipMisc() {
        for (;;) {
            skipWs();
            if (startsWith("<?")) skipPast("?>");
            else if (startsWith("<!--")) skipPast("-->");
            else if (startsWith("<!")) skipPast(">");
            else return;
        }
    }
    static std::string localName(const std::string& n) {
        size_t c = n.find(':');
        return c == std::string::npos ? n : n.substr(c + 1);
    }
    std::string name() {
        size_t b = pos_;
        while (pos_ < s_.size() && !std::isspace((unsigned char)s_[pos_]) && s_[pos_] != '>' && s_[pos_] != '/' && s_[pos_] != '=')
            ++pos_;
        if (b == pos_) fail("expected a name");
        return s_.substr(b, pos_ - b);
    }
    static std::string decode(const std::string& t) {
        std::string out;
        out.reserve(t.size());
        for (size_t i = 0; i < t.size(); ++i) {
            if (t[i] != '&') {
                out += t[i];
                continue;
            }
            size_t e = t.find(';', i);
            if (e == std::string::npos) {
                out += t[i];
                continue;
            }
            const std::string ent = t.substr(i + 1, e - i - 1);
            if (ent == "lt") out += '<';
            else if (ent == "gt") out += '>';
            else if (ent == "amp") out += '&';
            else if (ent == "quot") out += '"';
            else if (ent == "apos") out += '\'';
            else if (!ent.empty() && ent[0] == '#') {
                long v = ent.size() > 1 && (ent[1] == 'x' || ent[1] == 'X') ? std::strtol(ent.c_str() + 2, nullptr, 16)
                                                                           : std::strtol(ent.c_str() + 1, nullptr, 10);
                out += v < 128 ? (char)v : '?';
            } else {
                out += t.substr(i, e - i + 1);
            }
            i = e;
        }
        return out;
    }
    std::unique_ptr<XmlNode> element() {
        ++pos_;  // '<'
        auto n = std::make_unique<XmlNode>();
        n->tag = localName(name());
        for (;;) {
            skipWs();
            if (pos_ >= s_.size()) fail("unterminated start tag");
            if (s_[pos_] == '/') {
                if (pos_ + 1 >= s_.size() || s_[pos_ + 1] != '>') fail("bad empty-element tag");
                pos_ += 2;
                return n;
            }
            if (s_[pos_] == '>') {
                ++pos_;
                break;
            }
            std::string an = localName(name());
            skipWs();
            if (pos_ >= s_.size() || s_[pos_] != '=') fail("expected '=' after attribute " + an);
            ++pos_;
            skipWs();
            if (pos_ >= s_.size() || (s_[pos_] != '"' && s_[pos_] != '\'')) fail("expected a quoted attribute value");
            const char q = s_[pos_++];
            size_t e = s_.find(q, pos_);
            if (e == std::string::npos) fail("unterminated attribute value");
            n->attrs.emplace_back(an, decode(s_.substr(pos_, e - pos_)));
            pos_ = e + 1;
        }
        // content
        for (;;) {
            size_t lt = s_.find('<', pos_);
            if (lt == std::string::npos) fail("unterminated element " + n->tag);
            n->text += decode(s_.substr(pos_, lt - pos_));
            pos_ = lt;
            if (startsWith("</")) {
                pos_ += 2;
                const std::string end = localName(name());
                if (end != n->tag) fail("mismatched end tag </" + end + "> for <" + n->tag + ">");
                skipWs();
                if (pos_ >= s_.size() || s_[pos_] != '>') fail("bad end tag");
                ++pos_;
                return n;
            }
            if (startsWith("<!--")) {
                skipPast("-->");
                continue;
            }
            if (startsWith("<![CDATA[")) {
                pos_ += 9;
                size_t e = s_.find("]]>", pos_);
                if (e == std::string::npos) fail("unterminated CDATA");
                n->text += s_.substr(pos_, e - pos_);
                pos_ = e + 3;
                continue;
            }
            if (startsWith("<?")) {
                skipPast("?>");
                continue;
            }
            n->kids.push_back(element());
        }
    }

    const std::string& s_;
    size_t pos_ = 0;
};

std::string readFile(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw ColladaError("cannot open " + path);
    std::ostringstream ss;
    ss << f.rdbuf();
    return ss.str();
}

std::vector<float> floats(const std::string& text) {
    std::vector<float> v;
    const char* p = text.c_str();
    for (;;) {
        while (*p && std::isspace((unsigned char)*p)) ++p;
        if (!*p) break;
        char* e = nullptr;
        float x = std::strtof(p, &e);
        if (e == p) throw ColladaError("bad number in float list");
        v.push_back(x);
        p = e;
    }
    return v;
}

std::vector<long> ints(const std::string& text) {
    std::vector<long> v;
    const char* p = text.c_str();
    for (;;) {
        while (*p && std::isspace((unsigned char)*p)) ++p;
        if (!*p) break;
        char* e = nullptr;
        long x = std::strtol(p, &e, 10);
        if (e == p) throw ColladaError("bad number in index list");
        v.push_back(x);
        p = e;
    }
    return v;
}

std::string stripHash(const std::string& u) { return !u.empty() && u[0] == '#' ? u.substr(1) : u; }

// ---- JSON (the subset material files use) --------------------------------------------------------
struct Json {
    enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<Json> arr;
    std::vector<std::pair<std::string, Json>> obj;  // insertion order
};

class JsonReader {
  public:
    explicit JsonReader(const std::string& s) : s_(s) {}
    Json document() {
        Json v = value();
        ws();
        if (pos_ != s_.size()) fail("trailing characters");
        return v;
    }

  private:
    [[noreturn]] void fail(const std::string& w) const { throw ColladaError("JSON: " + w + " at byte " + std::to_string(pos_)); }
    void ws() {
        while (pos_ < s_.size() && std::isspace((unsigned char)s_[pos_])) ++pos_;
    }
    std::string string() {
        if (s_[pos_] != '"') fail("expected a string");
        ++pos_;
        std::string out;
        while (pos_ < s_.size() && s_[pos_] != '"') {
            char c = s_[pos_++];
            if (c == '\\') {
                if (pos_ >= s_.size()) fail("bad escape");
                char e = s_[pos_++];
                switch (e) {
                    case 'n': out += '\n'; break;
                    case 't': out += '\t'; break;
                    case 'r': out += '\r'; break;
                    case 'b': out += '\b'; break;
                    case 'f': out += '\f'; break;
                    case 'u': {
                        if (pos_ + 4 > s_.size()) fail("bad \\u escape");
                        long v = std::strtol(s_.substr(pos_, 4).c_str(), nullptr, 16);
                        out += v < 128 ? (char)v : '?';
                        pos_ += 4;
                        break;
                    }
                    default: out += e;
                }
            } else {
                out += c;
            }
        }
        if (pos_ >= s_.size()) fail("unterminated string");
        ++pos_;
        return out;
    }
    Json value() {
        ws();
        if (pos_ >= s_.size()) fail("unexpected end");
        Json v;
        const char c = s_[pos_];
        if (c == '{') {
            v.kind = Json::Object;
            ++pos_;
            ws();
            if (pos_ < s_.size() && s_[pos_] == '}') {
                ++pos_;
                return v;
            }
            for (;;) {
                ws();
                std::string k = string();
                ws();
                if (pos_ >= s_.size() || s_[pos_] != ':') fail("expected ':'");
                ++pos_;
                v.obj.emplace_back(k, value());
                ws();
                if (pos_ < s_.size() && s_[pos_] == ',') {
                    ++pos_;
                    continue;
                }
                if (pos_ < s_.size() && s_[pos_] == '}') {
                    ++pos_;
                    return v;
                }
                fail("expected ',' or '}'");
            }
        }
        if (c == '[') {
            v.kind = Json::Array;
            ++pos_;
            ws();
            if (pos_ < s_.size() && s_[pos_] == ']') {
                ++pos_;
                return v;
            }
            for (;;) {
                v.arr.push_back(value());
                ws();
                if (pos_ < s_.size() && s_[pos_] == ',') {
                    ++pos_;
                    continue;
                }
                if (pos_ < s_.size() && s_[pos_] == ']') {
                    ++pos_;
                    return v;
                }
                fail("expected ',' or ']'");
            }
        }
        if (c == '"') {
            v.kind = Json::String;
            v.str = string();
            return v;
        }
        if (s_.compare(pos_, 4, "true") == 0) {
            v.kind = Json::Bool;
            v.b = true;
            pos_ += 4;
            return v;
        }
        if (s_.compare(pos_, 5, "false") == 0) {
            v.kind = Json::Bool;
            pos_ += 5;
            return v;
        }
        if (s_.compare(pos_, 4, "null") == 0) {
            pos_ += 4;
            return v;
        }
        char* e = nullptr;
        v.num = std::strtod(s_.c_str() + pos_, &e);
        if (e == s_.c_str() + pos_) fail("unexpected character");
        v.kind = Json::Number;
        pos_ = (size_t)(e - s_.c_str());
        return v;
    }

    const std::string& s_;
    size_t pos_ = 0;
};

float jnum(const Json& v, const std::string& key) {
    if (v.kind == Json::Number) return (float)v.num;
    if (v.kind == Json::Bool) return v.b ? 1.0f : 0.0f;
    throw ColladaError("material field '" + key + "' is not a number");
}

void jvec3(const Json& v, const std::string& key, float out[3]) {
    if (v.kind != Json::Array || v.arr.size() != 3) throw ColladaError("material field '" + key + "' is not a 3-vector");
    for (int k = 0; k < 3; ++k) out[k] = jnum(v.arr[k], key);
}

std::string dirOf(const std::string& path) {
    size_t s = path.find_last_of('/');
    return s == std::string::npos ? std::string(".") : path.substr(0, s);
}

bool fileExists(const std::string& path) {
    std::ifstream f(path);
    return (bool)f;
}

std::shared_ptr<Material> loadMaterialDepth(const std::string& path, int depth) {
    if (depth > 16) throw ColladaError("material 'basedOn' chain too deep at " + path);
    const Json d = JsonReader(readFile(path)).document();
    auto m = std::make_shared<Material>();
    if (d.kind != Json::Object) throw ColladaError("not a material object: " + path);
    const Json* type = nullptr;
    for (const auto& kv : d.obj)
        if (kv.first == "type") type = &kv.second;
    if (!type || type->kind != Json::String || type->str != "Material") return m;  // "Not a material": the default
    for (const auto& kv : d.obj)
        if (kv.first == "basedOn") {
            if (kv.second.kind != Json::String) throw ColladaError("'basedOn' is not a string in " + path);
            const std::string base = dirOf(path) + "/" + kv.second.str + ".rgmat.json";
            if (fileExists(base)) m->gpu = loadMaterialDepth(base, depth + 1)->gpu;
        }
    rg_material& g = m->gpu;
    for (const auto& kv : d.obj) {
        const std::string& k = kv.first;
        const Json& v = kv.second;
        if (k == "type" || k == "basedOn") continue;
        if (k == "diffuse") jvec3(v, k, g.diffuse);
        else if (k == "transparency") g.transparency = jnum(v, k);
        else if (k == "specular") jvec3(v, k, g.specular);
        else if (k == "reflectivity") g.reflectivity = jnum(v, k);
        else if (k == "roughness") g.roughness = jnum(v, k);
        else if (k == "ior") g.ior = jnum(v, k);
        else if (k == "effectId") g.effectId = (uint32_t)jnum(v, k);
        else if (k == "rayConsumption") g.rayConsumption = (uint32_t)jnum(v, k);
        else if (k == "emission") g.emission = jnum(v, k);
        // staticFriction / dynamicFriction belong to the physics material; other keys are ignored
    }
    return m;
}

// ---- Collada ------------------------------------------------------------------------------------
struct Source {
    std::vector<float> data;
    size_t stride = 1;
};

struct Input {
    std::string semantic, source;
    size_t offset = 0;
};

struct Primitive {
    std::string materialSymbol;
    std::vector<Input> inputs;
    std::vector<long> p;       // index tuples
    std::vector<long> vcount;  // corners per polygon (triangles: all 3)
};

struct Geometry {
    std::map<std::string, Source> sources;
    std::map<std::string, std::vector<Input>> vertices;  // <vertices id> -> its inputs
    std::vector<Primitive> prims;
};

struct Node {
    std::string name;
    mat4 matrix;  // column-major
    std::vector<std::pair<std::string, std::map<std::string, std::string>>> geometries;  // (geometry id, symbol -> material id)
    std::vector<Node> children;
};

mat4 fromRowMajor(const std::vector<float>& v, size_t at) {
    mat4 m;
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) m.m[c][r] = v[at + 4 * r + c];
    return m;
}

mat4 rotationAxisAngle(float x, float y, float z, float deg) {
    const float len = std::sqrt(x * x + y * y + z * z);
    mat4 m;
    if (len == 0.0f) return m;
    x /= len;
    y /= len;
    z /= len;
    const float a = deg * 3.14159265358979f / 180.0f, c = std::cos(a), s = std::sin(a), t = 1.0f - c;
    m.m[0][0] = t * x * x + c;     m.m[1][0] = t * x * y - s * z; m.m[2][0] = t * x * z + s * y;
    m.m[0][1] = t * x * y + s * z; m.m[1][1] = t * y * y + c;     m.m[2][1] = t * y * z - s * x;
    m.m[0][2] = t * x * z - s * y; m.m[1][2] = t * y * z + s * x; m.m[2][2] = t * z * z + c;
    return m;
}

Node readNode(const XmlNode& x) {
    Node n;
    n.name = x.attrOr("name", x.attrOr("id", ""));
    for (const auto& k : x.kids) {
        const XmlNode& e = *k;
        if (e.tag == "matrix") {
            auto v = floats(e.text);
            if (v.size() != 16) throw ColladaError("node " + n.name + ": <matrix> needs 16 numbers");
            n.matrix = n.matrix * fromRowMajor(v, 0);
        } else if (e.tag == "translate") {
            auto v = floats(e.text);
            if (v.size() != 3) throw ColladaError("node " + n.name + ": <translate> needs 3 numbers");
            mat4 t;
            t.m[3][0] = v[0];
            t.m[3][1] = v[1];
            t.m[3][2] = v[2];
            n.matrix = n.matrix * t;
        } else if (e.tag == "rotate") {
            auto v = floats(e.text);
            if (v.size() != 4) throw ColladaError("node " + n.name + ": <rotate> needs 4 numbers");
            n.matrix = n.matrix * rotationAxisAngle(v[0], v[1], v[2], v[3]);
        } else if (e.tag == "scale") {
            auto v = floats(e.text);
            if (v.size() != 3) throw ColladaError("node " + n.name + ": <scale> needs 3 numbers");
            mat4 s;
            s.m[0][0] = v[0];
            s.m[1][1] = v[1];
            s.m[2][2] = v[2];
            n.matrix = n.matrix * s;
        } else if (e.tag == "lookat" || e.tag == "skew") {
            throw ColladaError("node " + n.name + ": <" + e.tag + "> transforms are not supported");
        } else if (e.tag == "instance_geometry") {
            std::map<std::string, std::string> bind;
            if (const XmlNode* bm = e.child("bind_material"))
                if (const XmlNode* tc = bm->child("technique_common"))
                    for (const XmlNode* im : tc->children("instance_material"))
                        bind[im->attrOr("symbol", "")] = stripHash(im->attrOr("target", ""));
            n.geometries.emplace_back(stripHash(e.attrOr("url", "")), bind);
        } else if (e.tag == "node") {
            n.children.push_back(readNode(e));
        } else if (e.tag == "instance_node") {
            throw ColladaError("node " + n.name + ": <instance_node> is not supported");
        }
    }
    return n;
}

Geometry readGeometry(const XmlNode& g) {
    Geometry out;
    const XmlNode* mesh = g.child("mesh");
    if (!mesh) throw ColladaError("geometry " + g.attrOr("id", "") + " has no <mesh>");
    for (const XmlNode* s : mesh->children("source")) {
        Source src;
        if (const XmlNode* fa = s->child("float_array")) src.data = floats(fa->text);
        if (const XmlNode* tc = s->child("technique_common"))
            if (const XmlNode* acc = tc->child("accessor")) src.stride = (size_t)std::max(1L, std::strtol(acc->attrOr("stride", "1").c_str(), nullptr, 10));
        out.sources[s->attrOr("id", "")] = std::move(src);
    }
    for (const XmlNode* v : mesh->children("vertices")) {
        std::vector<Input> ins;
        for (const XmlNode* in : v->children("input")) ins.push_back({in->attrOr("semantic", ""), stripHash(in->attrOr("source", "")), 0});
        out.vertices[v->attrOr("id", "")] = ins;
    }
    for (const auto& k : mesh->kids) {
        const XmlNode& e = *k;
        if (e.tag != "triangles" && e.tag != "polylist" && e.tag != "polygons") {
            if (e.tag == "lines" || e.tag == "linestrips" || e.tag == "trifans" || e.tag == "tristrips")
                throw ColladaError("<" + e.tag + "> primitives are not supported");
            continue;
        }
        Primitive p;
        p.materialSymbol = e.attrOr("material", "");
        for (const XmlNode* in : e.children("input"))
            p.inputs.push_back({in->attrOr("semantic", ""), stripHash(in->attrOr("source", "")),
                                (size_t)std::strtol(in->attrOr("offset", "0").c_str(), nullptr, 10)});
        size_t stride = 0;
        for (const auto& in : p.inputs) stride = std::max(stride, in.offset + 1);
        if (stride == 0) throw ColladaError("primitive without inputs");
        if (e.tag == "polygons") {
            for (const XmlNode* pe : e.children("p")) {
                auto v = ints(pe->text);
                p.vcount.push_back((long)(v.size() / stride));
                p.p.insert(p.p.end(), v.begin(), v.end());
            }
        } else {
            if (const XmlNode* pe = e.child("p")) p.p = ints(pe->text);
            if (e.tag == "polylist") {
                if (const XmlNode* vc = e.child("vcount")) p.vcount = ints(vc->text);
            } else {
                p.vcount.assign(p.p.size() / stride / 3, 3);
            }
        }
        out.prims.push_back(std::move(p));
    }
    return out;
}

// loadMesh of one primitive (entity.cpp:32-64): one vertex per face corner
std::shared_ptr<Mesh> primitiveMesh(const Geometry& g, const Primitive& p, uint32_t matIndex) {
    const Source* pos = nullptr;
    const Source* nrm = nullptr;
    size_t posOff = 0, nrmOff = 0;
    size_t stride = 0;
    for (const auto& in : p.inputs) stride = std::max(stride, in.offset + 1);
    for (const auto& in : p.inputs) {
        if (in.semantic == "VERTEX") {
            auto vit = g.vertices.find(in.source);
            if (vit == g.vertices.end()) throw ColladaError("unknown <vertices> " + in.source);
            for (const auto& vi : vit->second) {
                auto sit = g.sources.find(vi.source);
                if (sit == g.sources.end()) throw ColladaError("unknown source " + vi.source);
                if (vi.semantic == "POSITION") {
                    pos = &sit->second;
                    posOff = in.offset;
                } else if (vi.semantic == "NORMAL") {
                    nrm = &sit->second;
                    nrmOff = in.offset;
                }
            }
        } else if (in.semantic == "NORMAL") {
            auto sit = g.sources.find(in.source);
            if (sit == g.sources.end()) throw ColladaError("unknown source " + in.source);
            nrm = &sit->second;
            nrmOff = in.offset;
        }
    }
    if (!pos) throw ColladaError("primitive without positions");
    if (!nrm) throw ColladaError("primitive without normals (the reference reads aiMesh::mNormals unconditionally)");
    if (pos->stride < 3 || nrm->stride < 3) throw ColladaError("positions / normals need 3 components");
    auto fetch = [&](const Source& s, long idx, float out[3]) {
        if (idx < 0 || (size_t)idx * s.stride + 3 > s.data.size()) throw ColladaError("index out of range");
        const size_t at = (size_t)idx * s.stride;
        out[0] = s.data[at];
        out[1] = s.data[at + 1];
        out[2] = s.data[at + 2];
    };
    auto corner = [&](size_t c) {
        rg_vertex v;
        std::memset(&v, 0, sizeof v);
        const size_t base = c * stride;
        if (base + stride > p.p.size()) throw ColladaError("<p> shorter than its primitive count");
        fetch(*pos, p.p[base + posOff], v.position);
        fetch(*nrm, p.p[base + nrmOff], v.normal);
        v.matIndex = matIndex;
        return v;
    };
    auto mesh = std::make_shared<Mesh>();
    size_t c0 = 0;
    for (long n : p.vcount) {
        if (n < 3) {  // degenerate polygon: skipped, as the triangulation step drops it
            c0 += (size_t)std::max(0L, n);
            continue;
        }
        for (long k = 1; k + 1 < n; ++k) {  // fan around the first corner
            const uint32_t b = (uint32_t)mesh->vertices.size();
            mesh->vertices.push_back(corner(c0));
            mesh->vertices.push_back(corner(c0 + (size_t)k));
            mesh->vertices.push_back(corner(c0 + (size_t)k + 1));
            mesh->indices.insert(mesh->indices.end(), {b, b + 1, b + 2});
        }
        c0 += (size_t)n;
    }
    return mesh;
}

void merge(Mesh& into, const Mesh& other) {  // render/mesh.cpp:52-62
    const uint32_t off = (uint32_t)into.vertices.size();
    for (uint32_t i : other.indices) into.indices.push_back(i + off);
    into.vertices.insert(into.vertices.end(), other.vertices.begin(), other.vertices.end());
}

}  // namespace

Transform transformFromMat4(const mat4& m) {
    Transform t;
    t.position = vec3(m.m[3][0], m.m[3][1], m.m[3][2]);
    vec3 col[3];
    float s[3];
    for (int i = 0; i < 3; ++i) {
        col[i] = vec3(m.m[i][0], m.m[i][1], m.m[i][2]);
        s[i] = std::sqrt(dot(col[i], col[i]));
    }
    if (s[0] == 0.0f || s[1] == 0.0f || s[2] == 0.0f) throw ColladaError("singular node transform");
    vec3 r[3] = {col[0] * (1.0f / s[0]), col[1] * (1.0f / s[1]), col[2] * (1.0f / s[2])};
    if (dot(r[0], cross(r[1], r[2])) < 0.0f) {  // mirrored basis: negate scale and basis
        for (int i = 0; i < 3; ++i) {
            s[i] = -s[i];
            r[i] = -r[i];
        }
    }
    t.scaling = vec3(s[0], s[1], s[2]);
    // rotation matrix R with columns r[i] -> unit quaternion (largest-component method)
    const float R00 = r[0].x, R11 = r[1].y, R22 = r[2].z;
    const float R10 = r[0].y, R20 = r[0].z, R01 = r[1].x, R21 = r[1].z, R02 = r[2].x, R12 = r[2].y;
    quat q;
    const float tr = R00 + R11 + R22;
    if (tr > 0.0f) {
        const float k = std::sqrt(tr + 1.0f) * 2.0f;
        q.w = 0.25f * k;
        q.x = (R21 - R12) / k;
        q.y = (R02 - R20) / k;
        q.z = (R10 - R01) / k;
    } else if (R00 > R11 && R00 > R22) {
        const float k = std::sqrt(1.0f + R00 - R11 - R22) * 2.0f;
        q.w = (R21 - R12) / k;
        q.x = 0.25f * k;
        q.y = (R01 + R10) / k;
        q.z = (R02 + R20) / k;
    } else if (R11 > R22) {
        const float k = std::sqrt(1.0f + R11 - R00 - R22) * 2.0f;
        q.w = (R02 - R20) / k;
        q.x = (R01 + R10) / k;
        q.y = 0.25f * k;
        q.z = (R12 + R21) / k;
    } else {
        const float k = std::sqrt(1.0f + R22 - R00 - R11) * 2.0f;
        q.w = (R10 - R01) / k;
        q.x = (R02 + R20) / k;
        q.y = (R12 + R21) / k;
        q.z = 0.25f * k;
    }
    t.rotation = q;
    return t;
}

std::shared_ptr<Material> loadMaterialFile(const std::string& path) { return loadMaterialDepth(path, 0); }

std::shared_ptr<Entity> loadColladaEntity(const std::string& name, const std::string& daePath, const std::string& materialsDir,
                                          ColladaInfo* info) {
    const std::string src = readFile(daePath);
    const auto doc = XmlReader(src).document();
    if (doc->tag != "COLLADA") throw ColladaError(daePath + " is not a Collada document");

    // materials, in id order; each with the name it is loaded by
    std::map<std::string, std::string> matNameById;
    if (const XmlNode* lm = doc->child("library_materials"))
        for (const XmlNode* m : lm->children("material")) {
            const std::string id = m->attrOr("id", "");
            matNameById[id] = m->attrOr("name", id);
        }
    std::vector<std::string> ids, names;
    for (const auto& kv : matNameById) {
        ids.push_back(kv.first);
        names.push_back(kv.second);
    }
    if (ids.empty()) {  // the importer's default material
        ids.push_back("");
        names.push_back("DefaultMaterial");
    }
    std::map<std::string, uint32_t> matIndex;
    for (uint32_t k = 0; k < ids.size(); ++k) matIndex[ids[k]] = k;

    std::map<std::string, Geometry> geometries;
    if (const XmlNode* lg = doc->child("library_geometries"))
        for (const XmlNode* g : lg->children("geometry")) geometries[g->attrOr("id", "")] = readGeometry(*g);

    const XmlNode* lvs = doc->child("library_visual_scenes");
    if (!lvs) throw ColladaError(daePath + " has no visual scene");
    const XmlNode* vs = nullptr;
    if (const XmlNode* sc = doc->child("scene"))
        if (const XmlNode* ivs = sc->child("instance_visual_scene")) {
            const std::string want = stripHash(ivs->attrOr("url", ""));
            for (const XmlNode* v : lvs->children("visual_scene"))
                if (v->attrOr("id", "") == want) vs = v;
        }
    if (!vs) vs = lvs->child("visual_scene");
    if (!vs) throw ColladaError(daePath + " has no visual scene");

    std::vector<std::shared_ptr<Material>> materials;
    if (!materialsDir.empty())
        for (const auto& n : names) {
            const std::string p = materialsDir + "/" + n + ".rgmat.json";
            materials.push_back(fileExists(p) ? loadMaterialFile(p) : std::make_shared<Material>());
        }

    // collapseMeshes (entity.cpp:66-80): the node's meshes, then its descendants', merged
    std::function<void(const Node&, Mesh&)> collapse = [&](const Node& n, Mesh& out) {
        for (const auto& ig : n.geometries) {
            auto git = geometries.find(ig.first);
            if (git == geometries.end()) throw ColladaError("node " + n.name + ": unknown geometry " + ig.first);
            for (const Primitive& p : git->second.prims) {
                auto b = ig.second.find(p.materialSymbol);
                const std::string target = b != ig.second.end() ? b->second : p.materialSymbol;
                auto mi = matIndex.find(target);
                const uint32_t m = mi != matIndex.end() ? mi->second : 0u;
                merge(out, *primitiveMesh(git->second, p, m));
            }
        }
        for (const Node& c : n.children) collapse(c, out);
    };

    auto entity = std::make_shared<Entity>(name);
    for (const XmlNode* xn : vs->children("node")) {
        const Node n = readNode(*xn);
        auto model = std::make_shared<Model>();
        model->mesh = std::make_shared<Mesh>();
        collapse(n, *model->mesh);
        model->materials = materials;
        auto child = entity->emplaceChild(n.name);
        child->setTransform(transformFromMat4(n.matrix));
        child->model = model;
    }
    if (info) {
        info->materialIds = ids;
        info->materialNames = names;
        const XmlNode* asset = doc->child("asset");
        const XmlNode* up = asset ? asset->child("up_axis") : nullptr;
        info->upAxis = up ? up->text : "Y_UP";
        while (!info->upAxis.empty() && std::isspace((unsigned char)info->upAxis.back())) info->upAxis.pop_back();
        while (!info->upAxis.empty() && std::isspace((unsigned char)info->upAxis.front())) info->upAxis.erase(0, 1);
    }
    return entity;
}

}  // namespace rg
