// gbpt_ingest.cpp -- scene ingest of the C ABI (include/gbpt.h): Wavefront
// OBJ + MTL geometry and materials, principled parameter files (.pbrdf) and
// the rectangular-light forms of the reference's scene scripts, gathered
// into one gb_scene_desc.
//
// Follows the reference's loading path:
//   add_objfile_to_flat_tri_list   hl-main.cpp:277-354   (triangles, per-corner
//                                  normals, group materials, fallback material)
//   convert_and_upload_materials   material-conversion.cpp:59-148 (a material
//                                  becomes principled when <dir>/<name>.pbrdf
//                                  exists, else Lambert with the MTL Kd)
//   PrincipledBRDFParameters::readFrom principledParameters.h:64-125 (keys)
//   light / add-rectlight          lights.scm:4-9, lights.cpp:84-96
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <new>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/gbpt.h"

struct gb_asset {
    std::vector<float> pos, nrm;  // 9 floats per triangle each
    std::vector<float> tc;        // 6 floats per triangle (vt of the corners, 0 where absent)
    std::vector<int> mat;
    std::vector<int> dtex;        // diffuse texture of each material (-1 = none)
    std::vector<std::vector<uint8_t>> tex_pixels;
    std::vector<gb_texture> textures;
    std::map<std::string, int> texture_index;  // by file path
    std::vector<gb_material> materials;
    std::vector<gb_principled_params> params;
    std::vector<gb_light> lights;
    std::vector<std::string> material_names;
    std::map<std::string, int> material_index;
    std::string err;
    int textures_ignored = 0;
};

namespace {

int fail(gb_asset* a, int code, const std::string& msg) {
    if (a) a->err = msg;
    return code;
}

std::string dir_of(const std::string& path) {
    size_t k = path.find_last_of('/');
    return k == std::string::npos ? std::string(".") : path.substr(0, k);
}

// Defaults of an unset principled field: 0, except opacity and transmission
// (principledParameters.h:23-24).
gb_principled_params principled_defaults() {
    gb_principled_params p;
    std::memset(&p, 0, sizeof(p));
    p.opacity = 1.0f;
    p.transmiss = 1.0f;
    return p;
}

// Whitespace-separated "key value..." pairs.  Unknown tokens are skipped, as
// the reference's reader skips them; a key glued to its value
// ("transmission0.0" in the bundled default.pbrdf) is therefore ignored
// there too and the field keeps its default here.
bool parse_pbrdf(const std::string& path, gb_principled_params* out) {
    std::ifstream in(path);
    if (!in) return false;
    gb_principled_params p = principled_defaults();
    struct Key {
        const char* name;
        float* dst;
        int n;
    };
    const Key keys[] = {{"color", p.color, 3},          {"metallic", &p.metallic, 1},
                        {"opacity", &p.opacity, 1},     {"subsurface", &p.subsurface, 1},
                        {"specular", &p.specular, 1},   {"roughness", &p.roughness, 1},
                        {"tintSpecular", &p.specular_tint, 1}, {"anisotropic", &p.anisotropic, 1},
                        {"sheen", &p.sheen, 1},         {"tintSheen", &p.sheen_tint, 1},
                        {"clearcoat", &p.clearcoat, 1}, {"glossClearcoat", &p.clearcoat_gloss, 1},
                        {"transmission", &p.transmiss, 1}};
    std::string tok;
    while (in >> tok) {
        for (const Key& k : keys) {
            if (tok != k.name) continue;
            for (int i = 0; i < k.n; ++i) {
                float v;
                if (!(in >> v)) return false;
                k.dst[i] = v;
            }
            break;
        }
    }
    *out = p;
    return true;
}

struct MtlEntry {
    float kd[3] = {0.0f, 0.0f, 0.0f};
    std::string texture;  // map_Kd, relative to the MTL file's directory
};

// Binary (P6) or ASCII (P3) PPM with maxval <= 255 as RGBA8, rows top first.
bool read_ppm(const std::string& path, std::vector<uint8_t>* rgba, int* w, int* h) {
    std::ifstream in(path, std::ios::binary);
    if (!in) return false;
    std::string magic;
    in >> magic;
    if (magic != "P6" && magic != "P3") return false;
    int vals[3], k = 0;
    while (k < 3 && in) {
        in >> std::ws;
        if (in.peek() == '#') { std::string c; std::getline(in, c); continue; }
        in >> vals[k++];
    }
    if (!in || k < 3 || vals[0] <= 0 || vals[1] <= 0 || vals[2] <= 0 || vals[2] > 255 ||
        (long long)vals[0] * vals[1] > (1ll << 26))
        return false;
    *w = vals[0];
    *h = vals[1];
    const size_t n = (size_t)vals[0] * vals[1];
    rgba->assign(4 * n, 255);
    if (magic == "P6") {
        in.get();  // the single whitespace after maxval
        std::vector<uint8_t> raw(3 * n);
        if (!in.read((char*)raw.data(), (std::streamsize)raw.size())) return false;
        for (size_t i = 0; i < n; ++i)
            for (int c = 0; c < 3; ++c) (*rgba)[4 * i + c] = raw[3 * i + c];
    } else {
        for (size_t i = 0; i < 3 * n; ++i) {
            int v;
            if (!(in >> v) || v < 0 || v > vals[2]) return false;
            (*rgba)[4 * (i / 3) + i % 3] = (uint8_t)v;
        }
    }
    if (vals[2] != 255)  // rescale to 0 .. 255
        for (size_t i = 0; i < 4 * n; ++i)
            if (i % 4 != 3) (*rgba)[i] = (uint8_t)(((*rgba)[i] * 255 + vals[2] / 2) / vals[2]);
    return true;
}

// Index of the texture in file `path`, loading it on first use; -1 when it
// cannot be read as PPM (counted in textures_ignored).
int texture_for(gb_asset* a, const std::string& path) {
    auto it = a->texture_index.find(path);
    if (it != a->texture_index.end()) return it->second;
    std::vector<uint8_t> px;
    int w = 0, h = 0;
    int idx = -1;
    if (read_ppm(path, &px, &w, &h)) {
        idx = (int)a->textures.size();
        a->tex_pixels.push_back(std::move(px));
        a->textures.push_back(gb_texture{w, h, nullptr});
        for (size_t k = 0; k < a->textures.size(); ++k) a->textures[k].rgba = a->tex_pixels[k].data();
    } else {
        a->textures_ignored++;
    }
    a->texture_index[path] = idx;
    return idx;
}

void parse_mtl(const std::string& path, std::map<std::string, MtlEntry>* out) {
    std::ifstream in(path);
    if (!in) return;
    std::string line, cur;
    while (std::getline(in, line)) {
        std::istringstream ls(line);
        std::string key;
        if (!(ls >> key) || key[0] == '#') continue;
        if (key == "newmtl") {
            ls >> cur;
            (*out)[cur] = MtlEntry();
        } else if (key == "Kd" && !cur.empty()) {
            MtlEntry& e = (*out)[cur];
            ls >> e.kd[0] >> e.kd[1] >> e.kd[2];
        } else if (key == "map_Kd" && !cur.empty()) {
            std::string f, tok;
            while (ls >> tok) f = tok;  // the file name is the last token (options come first)
            if (!f.empty()) (*out)[cur].texture = dir_of(path) + "/" + f;
        }
    }
}

// Index of material `name`, creating it on first use: principled when
// material_dir/<name>.pbrdf exists, else Lambert with the MTL diffuse colour.
int material_for(gb_asset* a, const std::string& name, const std::map<std::string, MtlEntry>& mtl,
                 const std::string& material_dir) {
    auto it = a->material_index.find(name);
    if (it != a->material_index.end()) return it->second;
    gb_material m;
    std::memset(&m, 0, sizeof(m));
    m.principled = -1;
    auto e = mtl.find(name);
    int tex = -1;
    if (e != mtl.end()) {
        for (int c = 0; c < 3; ++c) m.diffuse[c] = e->second.kd[c];
        if (!e->second.texture.empty()) tex = texture_for(a, e->second.texture);
    }
    gb_principled_params p;
    if (!material_dir.empty() && parse_pbrdf(material_dir + "/" + name + ".pbrdf", &p)) {
        m.principled = (int)a->params.size();
        a->params.push_back(p);
    }
    int idx = (int)a->materials.size();
    a->materials.push_back(m);
    a->dtex.push_back(tex);
    a->material_names.push_back(name);
    a->material_index[name] = idx;
    return idx;
}

int obj_index(int i, int n) { return i > 0 ? i - 1 : n + i; }

}  // namespace

extern "C" {

int gb_asset_create(gb_asset** out) {
    if (!out) return GB_ERR_INVALID;
    *out = new (std::nothrow) gb_asset();
    return *out ? GB_OK : GB_ERR_OOM;
}

void gb_asset_destroy(gb_asset* a) { delete a; }

const char* gb_asset_last_error(const gb_asset* a) { return a ? a->err.c_str() : "null asset"; }

int gb_read_pbrdf(const char* path, gb_principled_params* out) {
    if (!path || !out) return GB_ERR_INVALID;
    return parse_pbrdf(path, out) ? GB_OK : GB_ERR_INVALID;
}

int gb_asset_add_obj(gb_asset* a, const char* obj_path, const char* material_dir, const float* trafo) {
    if (!a || !obj_path) return fail(a, GB_ERR_INVALID, "null argument");
    std::ifstream in(obj_path);
    if (!in) return fail(a, GB_ERR_INVALID, std::string("cannot open ") + obj_path);
    const std::string mdir = material_dir ? material_dir : "";
    // the fallback material of objects without one (hl-main.cpp:296-302)
    if (a->materials.empty()) {
        gb_material fb;
        std::memset(&fb, 0, sizeof(fb));
        fb.diffuse[0] = 1.0f;
        fb.principled = -1;
        a->materials.push_back(fb);
        a->dtex.push_back(-1);
        a->material_names.push_back("gi/fallback");
        a->material_index["gi/fallback"] = 0;
    }
    float M[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    if (trafo) std::memcpy(M, trafo, sizeof(M));
    // normal matrix: inverse transpose of the upper 3x3 (cofactors / det)
    double A[9] = {M[0], M[1], M[2], M[4], M[5], M[6], M[8], M[9], M[10]};
    double cof[9] = {A[4] * A[8] - A[5] * A[7], A[5] * A[6] - A[3] * A[8], A[3] * A[7] - A[4] * A[6],
                     A[2] * A[7] - A[1] * A[8], A[0] * A[8] - A[2] * A[6], A[1] * A[6] - A[0] * A[7],
                     A[1] * A[5] - A[2] * A[4], A[2] * A[3] - A[0] * A[5], A[0] * A[4] - A[1] * A[3]};
    double det = A[0] * cof[0] + A[1] * cof[1] + A[2] * cof[2];
    if (!(std::fabs(det) > 0.0)) return fail(a, GB_ERR_INVALID, "singular transformation");
    if (det < 0.0)  // inverse transpose = cofactors / det: keep det's sign
        for (double& c : cof) c = -c;
    std::vector<float> v, vn, vt;
    std::map<std::string, MtlEntry> mtl;
    int cur_mat = 0;
    const size_t tri0 = a->mat.size();
    std::string line;
    int lineno = 0;
    while (std::getline(in, line)) {
        ++lineno;
        std::istringstream ls(line);
        std::string key;
        if (!(ls >> key) || key[0] == '#') continue;
        if (key == "v" || key == "vn") {
            double x, y, z;
            if (!(ls >> x >> y >> z)) return fail(a, GB_ERR_INVALID, "bad vertex at line " + std::to_string(lineno));
            std::vector<float>& dst = key == "v" ? v : vn;
            if (key == "v") {
                dst.push_back((float)(M[0] * x + M[1] * y + M[2] * z + M[3]));
                dst.push_back((float)(M[4] * x + M[5] * y + M[6] * z + M[7]));
                dst.push_back((float)(M[8] * x + M[9] * y + M[10] * z + M[11]));
            } else {
                double nx = cof[0] * x + cof[1] * y + cof[2] * z, ny = cof[3] * x + cof[4] * y + cof[5] * z,
                       nz = cof[6] * x + cof[7] * y + cof[8] * z;
                double l = std::sqrt(nx * nx + ny * ny + nz * nz);
                if (l > 0.0) { nx /= l; ny /= l; nz /= l; }
                dst.push_back((float)nx); dst.push_back((float)ny); dst.push_back((float)nz);
            }
        } else if (key == "vt") {
            double s_, t_ = 0.0;
            if (!(ls >> s_)) return fail(a, GB_ERR_INVALID, "bad texture coordinate at line " + std::to_string(lineno));
            ls >> t_;
            vt.push_back((float)s_);
            vt.push_back((float)t_);
        } else if (key == "mtllib") {
            std::string f;
            ls >> f;
            parse_mtl(dir_of(obj_path) + "/" + f, &mtl);
        } else if (key == "usemtl") {
            std::string name;
            ls >> name;
            // names the MTL does not define fall back (material(name) == -1 and no group material)
            cur_mat = mtl.count(name) ? material_for(a, name, mtl, mdir) : 0;
        } else if (key == "f") {
            std::vector<int> vi, ni, ti;
            std::string c;
            const int nv = (int)v.size() / 3, nn = (int)vn.size() / 3, nt = (int)vt.size() / 2;
            while (ls >> c) {
                int iv = 0, it = 0, in_ = 0;
                size_t s1 = c.find('/');
                iv = std::atoi(c.substr(0, s1).c_str());
                if (s1 != std::string::npos) {
                    size_t s2 = c.find('/', s1 + 1);
                    if (s2 != std::string::npos) {
                        if (s2 > s1 + 1) it = std::atoi(c.substr(s1 + 1, s2 - s1 - 1).c_str());
                        in_ = std::atoi(c.substr(s2 + 1).c_str());
                    } else if (s1 + 1 < c.size()) {
                        it = std::atoi(c.substr(s1 + 1).c_str());
                    }
                }
                int t_ = it ? obj_index(it, nt) : -1;
                if (it && (t_ < 0 || t_ >= nt))
                    return fail(a, GB_ERR_INVALID, "texture coordinate index out of range at line " + std::to_string(lineno));
                ti.push_back(t_);
                int a_ = obj_index(iv, nv);
                if (iv == 0 || a_ < 0 || a_ >= nv)
                    return fail(a, GB_ERR_INVALID, "vertex index out of range at line " + std::to_string(lineno));
                vi.push_back(a_);
                int b_ = in_ ? obj_index(in_, nn) : -1;
                if (in_ && (b_ < 0 || b_ >= nn))
                    return fail(a, GB_ERR_INVALID, "normal index out of range at line " + std::to_string(lineno));
                ni.push_back(b_);
            }
            if (vi.size() < 3) return fail(a, GB_ERR_INVALID, "face with fewer than 3 vertices at line " + std::to_string(lineno));
            for (size_t k = 1; k + 1 < vi.size(); ++k) {  // fan
                const int cv[3] = {vi[0], vi[k], vi[k + 1]};
                const int cn[3] = {ni[0], ni[k], ni[k + 1]};
                const int ct[3] = {ti[0], ti[k], ti[k + 1]};
                for (int j = 0; j < 3; ++j) {
                    a->tc.push_back(ct[j] >= 0 ? vt[2 * ct[j]] : 0.0f);
                    a->tc.push_back(ct[j] >= 0 ? vt[2 * ct[j] + 1] : 0.0f);
                }
                float P[9];
                for (int j = 0; j < 3; ++j)
                    for (int d = 0; d < 3; ++d) P[3 * j + d] = v[3 * cv[j] + d];
                // geometric normal for corners without one
                float e1[3] = {P[3] - P[0], P[4] - P[1], P[5] - P[2]}, e2[3] = {P[6] - P[0], P[7] - P[1], P[8] - P[2]};
                double g[3] = {(double)e1[1] * e2[2] - (double)e1[2] * e2[1], (double)e1[2] * e2[0] - (double)e1[0] * e2[2],
                               (double)e1[0] * e2[1] - (double)e1[1] * e2[0]};
                double gl = std::sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
                if (gl > 0.0) { g[0] /= gl; g[1] /= gl; g[2] /= gl; }
                for (int j = 0; j < 3; ++j) {
                    for (int d = 0; d < 3; ++d) {
                        a->pos.push_back(P[3 * j + d]);
                        a->nrm.push_back(cn[j] >= 0 ? vn[3 * cn[j] + d] : (float)g[d]);
                    }
                }
                a->mat.push_back(cur_mat);
            }
        }
        // o / g / s lines carry nothing the path needs
    }
    if (a->mat.size() == tri0) return fail(a, GB_ERR_INVALID, std::string("no faces in ") + obj_path);
    return GB_OK;
}

int gb_asset_add_light(gb_asset* a, const gb_light* l) {
    if (!a || !l) return fail(a, GB_ERR_INVALID, "null argument");
    a->lights.push_back(*l);
    return GB_OK;
}

}  // extern "C"

namespace {

// Minimal s-expression reader for scene scripts: lists, strings, numbers,
// symbols and keywords; ';' starts a comment.
struct Sx {
    enum Kind { LIST, ATOM, STR } kind = ATOM;
    std::string text;
    std::vector<Sx> items;
};

bool read_sx(const std::string& s, size_t& i, Sx* out, int depth) {
    if (depth > 256) return false;
    auto skip = [&]() {
        while (i < s.size()) {
            if (std::isspace((unsigned char)s[i])) ++i;
            else if (s[i] == ';') { while (i < s.size() && s[i] != '\n') ++i; }
            else break;
        }
    };
    skip();
    if (i >= s.size()) return false;
    if (s[i] == '(') {
        ++i;
        out->kind = Sx::LIST;
        while (true) {
            skip();
            if (i >= s.size()) return false;
            if (s[i] == ')') { ++i; return true; }
            Sx c;
            if (!read_sx(s, i, &c, depth + 1)) return false;
            out->items.push_back(c);
        }
    }
    if (s[i] == '"') {
        size_t j = s.find('"', i + 1);
        if (j == std::string::npos) return false;
        out->kind = Sx::STR;
        out->text = s.substr(i + 1, j - i - 1);
        i = j + 1;
        return true;
    }
    if (s[i] == ')') return false;
    size_t j = i;
    while (j < s.size() && !std::isspace((unsigned char)s[j]) && s[j] != '(' && s[j] != ')' && s[j] != ';') ++j;
    out->kind = Sx::ATOM;
    out->text = s.substr(i, j - i);
    i = j;
    return true;
}

bool sx_numbers(const Sx& v, float* dst, int n) {
    // (list a b c) or a bare number
    if (v.kind == Sx::ATOM && n == 1) {
        char* e = nullptr;
        dst[0] = std::strtof(v.text.c_str(), &e);
        return e && *e == '\0' && !v.text.empty();
    }
    if (v.kind != Sx::LIST || v.items.empty() || v.items[0].text != "list" || (int)v.items.size() != n + 1) return false;
    for (int k = 0; k < n; ++k) {
        const Sx& it = v.items[k + 1];
        char* e = nullptr;
        dst[k] = std::strtof(it.text.c_str(), &e);
        if (it.kind != Sx::ATOM || !e || *e != '\0') return false;
    }
    return true;
}

// (light "name" :type :rect :color (list r g b) :pos (list ...) :dir (list ...)
//  :up (list ...) :dim (list w h)) anywhere in the tree.
void collect_lights(const Sx& x, std::vector<gb_light>* out, int* skipped, std::string* err) {
    if (x.kind != Sx::LIST) return;
    if (!x.items.empty() && x.items[0].kind == Sx::ATOM && x.items[0].text == "light") {
        std::map<std::string, const Sx*> kv;
        for (size_t k = 1; k + 1 < x.items.size(); ++k)
            if (x.items[k].kind == Sx::ATOM && !x.items[k].text.empty() && x.items[k].text[0] == ':')
                kv[x.items[k].text] = &x.items[k + 1];
        auto t = kv.find(":type");
        if (t == kv.end() || t->second->text != ":rect") { ++*skipped; return; }
        gb_light l;
        std::memset(&l, 0, sizeof(l));
        l.type = GB_LIGHT_RECT;
        l.power = -1.0f;  // add-rectlight's rule (lights.cpp:92)
        const char* names[5] = {":color", ":pos", ":dir", ":up", ":dim"};
        float* dst[5] = {l.col, l.center, l.dir, l.up, l.wh};
        const int n[5] = {3, 3, 3, 3, 2};
        for (int k = 0; k < 5; ++k) {
            auto f = kv.find(names[k]);
            if (f == kv.end() || !sx_numbers(*f->second, dst[k], n[k])) {
                *err = std::string("rect light without a numeric ") + names[k];
                return;
            }
        }
        out->push_back(l);
        return;
    }
    for (const Sx& c : x.items) collect_lights(c, out, skipped, err);
}

}  // namespace

extern "C" int gb_asset_add_lights(gb_asset* a, const char* script_path, int* skipped_lights) {
    if (!a || !script_path) return fail(a, GB_ERR_INVALID, "null argument");
    std::ifstream in(script_path);
    if (!in) return fail(a, GB_ERR_INVALID, std::string("cannot open ") + script_path);
    std::stringstream ss;
    ss << in.rdbuf();
    const std::string text = ss.str();
    std::vector<gb_light> found;
    int skipped = 0;
    std::string err;
    size_t i = 0;
    while (true) {
        size_t before = i;
        Sx x;
        if (!read_sx(text, i, &x, 0)) {
            // trailing whitespace / comments end the script; anything else is malformed
            size_t j = before;
            while (j < text.size() && (std::isspace((unsigned char)text[j]) || text[j] == ';')) {
                if (text[j] == ';') while (j < text.size() && text[j] != '\n') ++j;
                else ++j;
            }
            if (j < text.size()) return fail(a, GB_ERR_INVALID, "malformed script near offset " + std::to_string(j));
            break;
        }
        collect_lights(x, &found, &skipped, &err);
        if (!err.empty()) return fail(a, GB_ERR_INVALID, err);
    }
    a->lights.insert(a->lights.end(), found.begin(), found.end());
    if (skipped_lights) *skipped_lights = skipped;
    return GB_OK;
}

extern "C" int gb_asset_get_desc(const gb_asset* a, gb_scene_desc* d) {
    if (!a || !d) return GB_ERR_INVALID;
    d->num_triangles = (int)a->mat.size();
    d->positions = a->pos.data();
    d->normals = a->nrm.data();
    d->material_index = a->mat.data();
    d->num_materials = (int)a->materials.size();
    d->materials = a->materials.data();
    d->num_params = (int)a->params.size();
    d->params = a->params.empty() ? nullptr : a->params.data();
    d->num_lights = (int)a->lights.size();
    d->lights = a->lights.empty() ? nullptr : a->lights.data();
    bool any_tex = false;
    for (int t : a->dtex) any_tex = any_tex || t >= 0;
    d->num_textures = (int)a->textures.size();
    d->textures = a->textures.empty() ? nullptr : a->textures.data();
    d->texcoords = any_tex ? a->tc.data() : nullptr;
    d->diffuse_texture = any_tex ? a->dtex.data() : nullptr;
    return GB_OK;
}

extern "C" int gb_asset_material_name(const gb_asset* a, int index, const char** name) {
    if (!a || !name || index < 0 || index >= (int)a->material_names.size()) return GB_ERR_INVALID;
    *name = a->material_names[index].c_str();
    return GB_OK;
}
