// obj.cu — Wavefront OBJ input (host code): the role of
// Scene::load_obj_file_as_aggregate (src/rt/scene.cpp:441-453), with the
// import semantics of the loader the reference vendors (src/rt/obj-loader.cpp
// :163-227 import, :306-455 triangle corners, :456-498 vertex sharing,
// :500-544 material groups, :546-621 generated normals, :798-1123 the two
// passes, :1124-1290 materials), restated here:
//
//  * v / vt / vn lines give positions (3 floats), texture coordinates (2)
//    and normals (3); f lines give polygons in one of the forms v, v/vt,
//    v//vn, v/vt/vn (the first corner decides), split as a fan (0, i, i+1).
//  * Indices are 1-based; a negative index k resolves to k + count - 1,
//    where count is the number of such elements read so far (the loader's
//    rule, one below the OBJ convention's k + count).
//  * Corners become vertices in the order met; a corner reuses an earlier
//    vertex with the same position index whose whole record (position,
//    texture coordinate, normal) is bytewise equal, else it adds one.
//  * Triangles carry the material active at their face (usemtl; an unknown
//    name or none is material 0).  mtllib names a material file beside the
//    OBJ file (newmtl, Kd, Ns / 1000, d or 1 - Tr); without one, material 0
//    is the default (diffuse 0.8, shininess 0, alpha 1).
//  * Runs of consecutive triangles with one material are groups, ordered by
//    alpha, highest first (the loader's sort; groups of equal alpha keep
//    their order, as its sort does for the few groups of these models).
//  * A file without normals gets them from the faces: every vertex sums the
//    unnormalised cross products of its triangles, then is scaled by
//    1 / sqrtf(|n|^2).
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <new>
#include <string>
#include <vector>

#include "../../include/rt_cuda.h"
#include "ctx_internal.h"

struct rt_obj {
    std::vector<float> pos, nrm;        // 3 per vertex
    std::vector<uint32_t> idx;          // 3 per triangle
    std::vector<rt_obj_group> groups;
};

namespace {

#define fail rt::set_error

struct ObjMaterial {
    std::string name;
    float diffuse[3] = {0.8f, 0.8f, 0.8f};
    float shininess = 0.0f, alpha = 1.0f;
};

// One vertex record as the sharing rule compares it.
struct Corner {
    float pos[3], tc[2], nrm[3];
};

struct Reader {
    std::vector<float> v, vt, vn;
    std::vector<Corner> verts;
    std::map<int, std::vector<int>> by_pos;   // position index -> vertices made from it
    std::vector<uint32_t> idx;
    std::vector<int> tri_mat;
    std::vector<ObjMaterial> mats;
    std::map<std::string, int> mat_index;
    int active = 0;

    int vertex(int pv, int pt, int pn, int form) {
        Corner c;
        memset(&c, 0, sizeof(c));
        for (int k = 0; k < 3; ++k) c.pos[k] = v[3 * (size_t)pv + k];
        if (form == 1 || form == 3)
            for (int k = 0; k < 2; ++k) c.tc[k] = vt[2 * (size_t)pt + k];
        if (form == 2 || form == 3)
            for (int k = 0; k < 3; ++k) c.nrm[k] = vn[3 * (size_t)pn + k];
        std::vector<int>& list = by_pos[pv];
        for (int i : list)
            if (memcmp(&verts[i], &c, sizeof(Corner)) == 0) return i;
        verts.push_back(c);
        list.push_back((int)verts.size() - 1);
        return (int)verts.size() - 1;
    }
};

// Resolves a 1-based OBJ index (the loader's rule for negative ones).
int resolve(long k, size_t count) { return (int)(k < 0 ? k + (long)count - 1 : k - 1); }

// Parses "a", "a/b", "a//c" or "a/b/c" into up to three integers; returns
// the form (0 v, 1 v/vt, 2 v//vn, 3 v/vt/vn) or -1.
int corner_form(const char* t, long out[3]) {
    char* end = nullptr;
    out[0] = strtol(t, &end, 10);
    if (end == t) return -1;
    if (*end != '/') return 0;
    if (end[1] == '/') {
        const char* s = end + 2;
        out[2] = strtol(s, &end, 10);
        return end == s ? -1 : 2;
    }
    const char* s = end + 1;
    out[1] = strtol(s, &end, 10);
    if (end == s) return -1;
    if (*end != '/') return 1;
    s = end + 1;
    out[2] = strtol(s, &end, 10);
    return end == s ? -1 : 3;
}

bool read_materials(const std::string& path, Reader& R) {
    FILE* f = fopen(path.c_str(), "r");
    if (!f) return false;
    char line[1024];
    ObjMaterial* cur = nullptr;
    std::vector<ObjMaterial> mats;
    while (fgets(line, sizeof(line), f)) {
        char key[64] = {0};
        if (sscanf(line, "%63s", key) != 1) continue;
        const char* rest = line + (strstr(line, key) - line) + strlen(key);
        if (!strcmp(key, "newmtl")) {
            char name[512] = {0};
            sscanf(rest, "%511s", name);
            mats.emplace_back();
            mats.back().name = name;
            cur = &mats.back();
        } else if (cur && !strcmp(key, "Kd")) {
            sscanf(rest, "%f %f %f", &cur->diffuse[0], &cur->diffuse[1], &cur->diffuse[2]);
        } else if (cur && !strcmp(key, "Ns")) {
            sscanf(rest, "%f", &cur->shininess);
            cur->shininess /= 1000.0f;
        } else if (cur && !strcmp(key, "d")) {
            sscanf(rest, "%f", &cur->alpha);
        } else if (cur && !strcmp(key, "Tr")) {
            float tr = 0.f;
            sscanf(rest, "%f", &tr);
            cur->alpha = 1.0f - tr;
        }
    }
    fclose(f);
    if (mats.empty()) return false;
    R.mats = mats;
    R.mat_index.clear();
    for (size_t i = 0; i < R.mats.size(); ++i) R.mat_index[R.mats[i].name] = (int)i;
    return true;
}

int32_t parse(const char* path, rt_obj* out) {
    FILE* f = fopen(path, "r");
    if (!f) return fail(RT_ERR_INVALID, "rt_obj_load: cannot open %s", path);
    std::string dir = path;
    const size_t slash = dir.find_last_of("/\\");
    dir = slash == std::string::npos ? std::string() : dir.substr(0, slash + 1);
    Reader R;
    std::vector<char> buf(1 << 16);
    std::string line;
    bool bad = false;
    // material files first (the loader reads them in its first pass, so a
    // usemtl above its mtllib line still finds its material)
    while (fgets(buf.data(), (int)buf.size(), f)) {
        const char* s = buf.data();
        while (*s == ' ' || *s == '\t') ++s;
        if (!strncmp(s, "mtllib", 6)) {
            char name[512] = {0};
            sscanf(s + 6, "%511s", name);
            read_materials(dir + name, R);
        }
    }
    rewind(f);
    while (fgets(buf.data(), (int)buf.size(), f)) {
        line.assign(buf.data());
        while (!line.empty() && line.back() != '\n' && fgets(buf.data(), (int)buf.size(), f))
            line += buf.data();   // longer than the buffer
        const char* s = line.c_str();
        while (*s == ' ' || *s == '\t') ++s;
        if (s[0] == 'v' && (s[1] == ' ' || s[1] == '\t')) {
            float x = 0, y = 0, z = 0;
            sscanf(s + 2, "%f %f %f", &x, &y, &z);
            R.v.insert(R.v.end(), {x, y, z});
        } else if (s[0] == 'v' && s[1] == 't') {
            float a = 0, b = 0;
            sscanf(s + 2, "%f %f", &a, &b);
            R.vt.insert(R.vt.end(), {a, b});
        } else if (s[0] == 'v' && s[1] == 'n') {
            float x = 0, y = 0, z = 0;
            sscanf(s + 2, "%f %f %f", &x, &y, &z);
            R.vn.insert(R.vn.end(), {x, y, z});
        } else if (s[0] == 'f' && (s[1] == ' ' || s[1] == '\t')) {
            std::vector<int> poly;
            int form = -1;
            char tok[128];
            int used = 0;
            const char* p = s + 1;
            while (sscanf(p, "%127s%n", tok, &used) == 1) {
                p += used;
                long k[3] = {0, 0, 0};
                const int fm = corner_form(tok, k);
                if (fm < 0) break;
                if (form < 0) form = fm;
                if (fm != form) break;
                const int pv = resolve(k[0], R.v.size() / 3);
                const int pt = (form == 1 || form == 3) ? resolve(k[1], R.vt.size() / 2) : 0;
                const int pn = (form == 2 || form == 3) ? resolve(k[2], R.vn.size() / 3) : 0;
                if (pv < 0 || (size_t)pv >= R.v.size() / 3 ||
                    ((form == 1 || form == 3) && (pt < 0 || (size_t)pt >= R.vt.size() / 2)) ||
                    ((form == 2 || form == 3) && (pn < 0 || (size_t)pn >= R.vn.size() / 3))) {
                    bad = true;
                    break;
                }
                poly.push_back(R.vertex(pv, pt, pn, form));
            }
            if (bad) break;
            for (size_t i = 1; i + 1 < poly.size(); ++i) {
                R.idx.insert(R.idx.end(), {(uint32_t)poly[0], (uint32_t)poly[i], (uint32_t)poly[i + 1]});
                R.tri_mat.push_back(R.active);
            }
        } else if (!strncmp(s, "usemtl", 6)) {
            char name[512] = {0};
            sscanf(s + 6, "%511s", name);
            auto it = R.mat_index.find(name);
            R.active = it == R.mat_index.end() ? 0 : it->second;
        }
    }
    fclose(f);
    if (bad) return fail(RT_ERR_INVALID, "rt_obj_load: %s: face index out of range", path);
    if (R.mats.empty()) R.mats.emplace_back();   // the default material
    const size_t V = R.verts.size(), N = R.idx.size() / 3;
    if (V == 0 || N == 0) return fail(RT_ERR_INVALID, "rt_obj_load: %s has no faces", path);
    // generated normals when the file has none
    if (R.vn.empty()) {
        std::vector<float> acc(3 * V, 0.0f);
        for (size_t t = 0; t < N; ++t) {
            const Corner& a = R.verts[R.idx[3 * t]];
            const Corner& b = R.verts[R.idx[3 * t + 1]];
            const Corner& c = R.verts[R.idx[3 * t + 2]];
            float e1[3], e2[3];
            for (int k = 0; k < 3; ++k) {
                e1[k] = b.pos[k] - a.pos[k];
                e2[k] = c.pos[k] - a.pos[k];
            }
            const float n[3] = {(e1[1] * e2[2]) - (e1[2] * e2[1]), (e1[2] * e2[0]) - (e1[0] * e2[2]),
                                (e1[0] * e2[1]) - (e1[1] * e2[0])};
            for (int j = 0; j < 3; ++j)
                for (int k = 0; k < 3; ++k) acc[3 * (size_t)R.idx[3 * t + j] + k] += n[k];
        }
        for (size_t i = 0; i < V; ++i) {
            float* n = &acc[3 * i];
            const float len = 1.0f / sqrtf(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
            for (int k = 0; k < 3; ++k) R.verts[i].nrm[k] = n[k] * len;
        }
    }
    out->pos.resize(3 * V);
    out->nrm.resize(3 * V);
    for (size_t i = 0; i < V; ++i)
        for (int k = 0; k < 3; ++k) {
            out->pos[3 * i + k] = R.verts[i].pos[k];
            out->nrm[3 * i + k] = R.verts[i].nrm[k];
        }
    out->idx = R.idx;
    // groups: runs of one material, highest alpha first
    for (size_t t = 0; t < N; ++t) {
        if (t == 0 || R.tri_mat[t] != R.tri_mat[t - 1]) {
            const ObjMaterial& m = R.mats[(size_t)R.tri_mat[t] < R.mats.size() ? R.tri_mat[t] : 0];
            rt_obj_group g;
            memset(&g, 0, sizeof(g));
            g.first_triangle = (uint32_t)t;
            for (int k = 0; k < 3; ++k) g.diffuse[k] = m.diffuse[k];
            g.shininess = m.shininess;
            g.alpha = m.alpha;
            out->groups.push_back(g);
        }
        ++out->groups.back().triangle_count;
    }
    std::stable_sort(out->groups.begin(), out->groups.end(),
                     [](const rt_obj_group& a, const rt_obj_group& b) { return a.alpha > b.alpha; });
    return RT_OK;
}

}  // namespace

extern "C" {

int32_t rt_obj_load(const char* path, rt_obj** out) {
    if (!path || !out) return fail(RT_ERR_INVALID, "rt_obj_load: null argument");
    rt_obj* o = new (std::nothrow) rt_obj();
    if (!o) return fail(RT_ERR_OOM, "rt_obj_load: host allocation failed");
    const int32_t r = parse(path, o);
    if (r) {
        delete o;
        return r;
    }
    *out = o;
    return RT_OK;
}

int32_t rt_obj_info(const rt_obj* o, uint32_t* vertices, uint32_t* triangles, uint32_t* groups) {
    if (!o) return fail(RT_ERR_INVALID, "rt_obj_info: null model");
    if (vertices) *vertices = (uint32_t)(o->pos.size() / 3);
    if (triangles) *triangles = (uint32_t)(o->idx.size() / 3);
    if (groups) *groups = (uint32_t)o->groups.size();
    return RT_OK;
}

int32_t rt_obj_copy(const rt_obj* o, float* pos4, float* nrm4, uint32_t* indices,
                    rt_obj_group* groups) {
    if (!o) return fail(RT_ERR_INVALID, "rt_obj_copy: null model");
    const size_t V = o->pos.size() / 3;
    for (size_t i = 0; i < V; ++i)
        for (int k = 0; k < 4; ++k) {
            if (pos4) pos4[4 * i + k] = k < 3 ? o->pos[3 * i + k] : 0.0f;
            if (nrm4) nrm4[4 * i + k] = k < 3 ? o->nrm[3 * i + k] : 0.0f;
        }
    if (indices) memcpy(indices, o->idx.data(), sizeof(uint32_t) * o->idx.size());
    if (groups) memcpy(groups, o->groups.data(), sizeof(rt_obj_group) * o->groups.size());
    return RT_OK;
}

int32_t rt_obj_free(rt_obj* o) {
    delete o;
    return RT_OK;
}

}  // extern "C"
