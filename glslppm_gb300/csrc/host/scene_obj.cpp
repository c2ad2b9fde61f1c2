// Scene ingest: OBJ/MTL reading with the semantics of the reference loader (mesh.cpp), the light
// table (TMesh::PrepareLightSources) and the bounding boxes (TMesh::CalculateBBox).
//
// The reference behaviour kept here, because the triangle data it produces is the input of the
// shader path and the parity tests compare it word for word:
//  * lines are read in chunks of at most 79 characters (fgets with an 80-byte buffer,
//    mesh.cpp:137,139 and :209,262); a longer line continues as a new "line";
//  * every mtllib line's MTL file is read before any usemtl line is matched (the reference reads
//    them in a first pass over the file, mesh.cpp:138-149), so a usemtl may name a material of
//    an MTL file listed further down;
//  * an MTL material is appended when its "Ns" line is read (mesh.cpp:178-186); Ka/Kd/Ks carry
//    over from the previous material when a block omits them; "Ke" is read as Ka (:155);
//  * material and usemtl names keep their trailing characters (newline) and must match exactly
//    (mesh.cpp:146-150, 305-321);
//  * faces use their first three vertices (:325-327); a missing normal index on any face vertex
//    switches the whole mesh to face normals (:334-341, 645-651);
//  * normals are normalised when read (:272-276); positions are p*scale+offset (:632-634);
//  * the material classifier of mesh.cpp:520-611 (mirror/plastic/glossy/glass/light, diffuse
//    albedo x0.9, glass albedo square-rooted) and the packed glossiness of gpurt.cpp:126.
// The file is read once and its lines are parsed in parallel ranges (cut at line ends, each cut
// into the same 79-character chunks); materials and errors are resolved afterwards in file order.
// Deliberate differences, reported as errors instead of undefined behaviour: unreadable files,
// malformed faces and out-of-range indices (SPPM_ERR_IO), "sss" materials (SPPM_ERR_UNSUPPORTED).
// map_Kd textures are binary 8-bit PPM files (LoadPPM, mesh.cpp:37-54).  The MTL file is opened relative to the OBJ file's directory.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "scene_internal.h"
#include "sppm_texture.h"

using sppm::fail;
using sppm::V3;
using sppm::v3;

namespace {

struct MtlEntry {
    std::string name;  // includes the characters after "newmtl " up to the end of the chunk
    V3 ka{0, 0, 0}, kd{0, 0, 0}, ks{0, 0, 0};
    float ns = 0.0f;
    bool textured = false;
    int tex_w = 0, tex_h = 0;
    std::vector<uint8_t> texture;  // RGB8, rows top to bottom as the P6 file stores them
};

std::string dir_of(const char* path) {
    const char* slash = strrchr(path, '/');
    return slash ? std::string(path, slash - path + 1) : std::string();
}

// LoadPPM (mesh.cpp:37-54): binary P6, maximum value 255
int load_ppm(const std::string& path, MtlEntry& m) {
    FILE* fp = fopen(path.c_str(), "rb");
    if (!fp) return fail(SPPM_ERR_IO, "cannot open texture '%s'", path.c_str());
    int w = 0, h = 0, maxv = 0;
    const bool ok = fscanf(fp, "P6 %d %d %d", &w, &h, &maxv) == 3 && w > 0 && h > 0 && maxv == 255 &&
                    (long long)w * h <= (1ll << 28) && fgetc(fp) != EOF;
    if (!ok) {
        fclose(fp);
        return fail(SPPM_ERR_IO, "'%s' is not a binary 8-bit PPM (P6, 255)", path.c_str());
    }
    m.tex_w = w;
    m.tex_h = h;
    m.texture.resize((size_t)w * h * 3);
    const size_t got = fread(m.texture.data(), 1, m.texture.size(), fp);
    fclose(fp);
    if (got != m.texture.size()) return fail(SPPM_ERR_IO, "texture '%s' is truncated", path.c_str());
    return SPPM_OK;
}

bool starts_with(const char* line, const char* prefix) {
    return strncmp(line, prefix, strlen(prefix)) == 0;
}

// the text after the first `skip` characters, as std::string::erase(0, skip) leaves it
std::string tail(const char* line, size_t skip) {
    const size_t n = strlen(line);
    return skip < n ? std::string(line + skip) : std::string();
}

int read_mtl(const std::string& path, std::vector<MtlEntry>& out) {
    FILE* fp = fopen(path.c_str(), "r");
    if (!fp) return fail(SPPM_ERR_IO, "cannot open MTL file '%s'", path.c_str());
    MtlEntry cur;  // reused between blocks, as the reference reuses its TMaterial
    char line[81];
    while (fgets(line, 80, fp) != nullptr) {
        float r = 0, g = 0, b = 0, s = 0;
        if (starts_with(line, "newmtl")) {
            cur.name = tail(line, 7);
            cur.textured = false;
        } else if (starts_with(line, "Ka") || starts_with(line, "Ke")) {
            sscanf(tail(line, 3).c_str(), "%f %f %f", &r, &g, &b);
            cur.ka = v3(r, g, b);
        } else if (starts_with(line, "Kd")) {
            sscanf(tail(line, 3).c_str(), "%f %f %f", &r, &g, &b);
            cur.kd = v3(r, g, b);
        } else if (starts_with(line, "Ks")) {
            sscanf(tail(line, 3).c_str(), "%f %f %f", &r, &g, &b);
            cur.ks = v3(r, g, b);
        } else if (starts_with(line, "Ns")) {
            sscanf(tail(line, 3).c_str(), "%f", &s);
            cur.ns = s;
            out.push_back(cur);
        } else if (starts_with(line, "map_Kd")) {
            // the texture goes to the material last appended (mesh.cpp:117-123): a map_Kd line
            // belongs after the block's Ns line
            std::string name = tail(line, 7);
            if (!name.empty()) name.erase(name.size() - 1, 1);
            if (out.empty()) {
                fclose(fp);
                return fail(SPPM_ERR_IO, "'%s': map_Kd before any complete material", path.c_str());
            }
            out.back().textured = true;
            const int st = load_ppm(dir_of(path.c_str()) + name, out.back());
            if (st != SPPM_OK) {
                fclose(fp);
                return st;
            }
        }
    }
    fclose(fp);
    return SPPM_OK;
}

// "v", "v/t", "v//n", "v/t/n" -> indices; a missing field reads as 0 (atoi of an empty field)
void split_face_vertex(const char* word, int* vi, int* ti, int* ni) {
    std::string w(word);
    size_t a = w.find('/');
    std::string sv = w.substr(0, a), st, sn;
    if (a != std::string::npos) {
        size_t b = w.find('/', a + 1);
        st = w.substr(a + 1, b == std::string::npos ? std::string::npos : b - a - 1);
        if (b != std::string::npos) {
            // a third '/' would end the normal field, as the reference replaces every '/' by '\0'
            size_t c = w.find('/', b + 1);
            sn = w.substr(b + 1, c == std::string::npos ? std::string::npos : c - b - 1);
        }
    }
    *vi = atoi(sv.c_str());
    *ti = atoi(st.c_str());
    *ni = atoi(sn.c_str());
}


// CGPURT::CreateTextures packs g = 1 / ((2 / (1 - specularity))^2.71828 + 1) (gpurt.cpp:126)
float packed_glossiness(float specularity) {
    return 1.0f / (std::pow(2.0f / (1.0f - specularity), 2.71828f) + 1.0f);
}

}  // namespace

void sppm_mesh::finish_geometry() {
    // TMesh::CalculateBBox (mesh.cpp:437-453)
    bbox.init();
    tri_bbox.resize(num_triangles);
    tri_centroid.resize(num_triangles);
    for (uint32_t i = 0; i < num_triangles; i++) {
        const V3 p0 = pos(i, 0), p1 = pos(i, 1), p2 = pos(i, 2);
        tri_bbox[i].init();
        tri_bbox[i].expand(p0);
        tri_bbox[i].expand(p1);
        tri_bbox[i].expand(p2);
        tri_centroid[i] = (p0 + p1 + p2) * (1.0f / 3.0f);
        bbox.expand(p0);
        bbox.expand(p1);
        bbox.expand(p2);
    }
}

void sppm_mesh::prepare_lights() {
    // TMesh::PrepareLightSources (mesh.cpp:456-488)
    light_area = 0.0f;
    light_cdf.clear();
    light_triangles.clear();
    for (uint32_t i = 0; i < num_triangles; i++) {
        if (materials[material_ids[i]].brdf == -1) {
            const V3 e0 = pos(i, 1) - pos(i, 0);
            const V3 e1 = pos(i, 2) - pos(i, 0);
            const V3 c = sppm::cross3(e0, e1);
            const float a = 0.5f * sppm::sqrt_f32(sppm::dot3(c, c));
            light_cdf.push_back(a);
            light_triangles.push_back((int32_t)i);
            light_area += a;
        }
    }
    if (light_cdf.empty()) return;
    for (size_t i = 1; i < light_cdf.size(); i++) light_cdf[i] = light_cdf[i] + light_cdf[i - 1];
    for (size_t i = 0; i < light_cdf.size(); i++) light_cdf[i] = light_cdf[i] / light_area;
}

namespace {

// what one range of the file's lines holds, in file order
struct ObjPart {
    std::vector<float> v, n, t;
    std::vector<int> vind, nind, tind;  // per face vertex (0-based; -1 for a missing index)
    uint32_t faces = 0;
    bool no_normals = false, no_texcoords = false;
    // mtllib and usemtl lines (resolved in file order afterwards: reading an MTL file appends
    // materials that later usemtl lines match) and the first malformed face
    struct Event {
        uint32_t face;  // faces of this part before the line
        int kind;       // 0 mtllib, 1 usemtl, 2 malformed face
        std::string name;
    };
    std::vector<Event> events;
};

// one fgets chunk of the reference's loop (mesh.cpp:209-345); false after a malformed face
bool parse_obj_line(const char* line, ObjPart& P) {
    if (starts_with(line, "mtllib")) {
        std::string name = tail(line, 7);
        if (!name.empty()) name.erase(name.size() - 1, 1);  // the reference drops the last character
        P.events.push_back({P.faces, 0, name});
    }
    if (line[0] == 'v') {
        if (line[1] == 'n') {
            float x = 0, y = 0, z = 0;
            sscanf(&line[2], "%f %f %f", &x, &y, &z);
            const float l = sppm::sqrt_f32(x * x + y * y + z * z);
            P.n.push_back(x / l);
            P.n.push_back(y / l);
            P.n.push_back(z / l);
        } else if (line[1] == 't') {
            float a = 0, b = 0;
            sscanf(&line[2], "%f %f", &a, &b);
            P.t.push_back(a);
            P.t.push_back(b);
        } else {
            float x = 0, y = 0, z = 0;
            sscanf(&line[1], "%f %f %f", &x, &y, &z);
            P.v.push_back(x);
            P.v.push_back(y);
            P.v.push_back(z);
        }
    }
    if (starts_with(line, "usemtl")) {
        P.events.push_back({P.faces, 1, tail(line, 7)});
    } else if (line[0] == 'f') {
        char w[3][32];
        if (sscanf(&line[1], "%31s %31s %31s", w[0], w[1], w[2]) != 3) {
            P.events.push_back({P.faces, 2, std::string()});
            return false;
        }
        for (int k = 0; k < 3; k++) {
            int vi, ti, ni;
            split_face_vertex(w[k], &vi, &ti, &ni);
            P.vind.push_back(vi - 1);
            if (ni) P.nind.push_back(ni - 1);
            else {
                P.nind.push_back(-1);
                P.no_normals = true;
            }
            if (ti) P.tind.push_back(ti - 1);
            else {
                P.tind.push_back(-1);
                P.no_texcoords = true;
            }
        }
        P.faces++;
    }
    return true;
}

// the lines of buf[begin, end) (begin at a line start), cut into chunks of at most 79 characters
// the way fgets(line, 80, fp) cuts them
void parse_obj_range(const char* buf, size_t begin, size_t end, ObjPart& P) {
    char line[81];
    size_t p = begin;
    while (p < end) {
        const char* nl = static_cast<const char*>(memchr(buf + p, '\n', end - p));
        const size_t stop = nl ? (size_t)(nl - buf) + 1 : end;  // past the newline
        while (p < stop) {
            const size_t len = std::min<size_t>(79, stop - p);
            memcpy(line, buf + p, len);
            line[len] = '\0';
            p += len;
            if (!parse_obj_line(line, P)) return;
        }
    }
}

}  // namespace

extern "C" int sppm_mesh_load_obj(const char* path, const float offset[3], float scale, sppm_mesh** out) {
    if (!path || !offset || !out) return fail(SPPM_ERR_ARG, "sppm_mesh_load_obj: null argument");
    *out = nullptr;
    FILE* fp = fopen(path, "rb");
    if (!fp) return fail(SPPM_ERR_IO, "cannot open OBJ file '%s'", path);
    std::vector<char> buf;
    {
        char block[1 << 16];
        size_t got;
        while ((got = fread(block, 1, sizeof block, fp)) > 0) buf.insert(buf.end(), block, block + got);
    }
    fclose(fp);
    // fgets stops at a NUL byte's line as text functions see it: keep the text before the first
    const size_t size = std::find(buf.begin(), buf.end(), '\0') - buf.begin();

    // ranges of whole lines, parsed in parallel
    unsigned threads = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    if (size < (4u << 20)) threads = 1;
    std::vector<size_t> cut(threads + 1, size);
    cut[0] = 0;
    for (unsigned k = 1; k < threads; k++) {
        size_t c = std::max(cut[k - 1], size * k / threads);
        const char* nl = c < size ? static_cast<const char*>(memchr(buf.data() + c, '\n', size - c)) : nullptr;
        cut[k] = nl ? (size_t)(nl - buf.data()) + 1 : size;
    }
    std::vector<ObjPart> parts(threads);
    {
        std::vector<std::thread> pool;
        for (unsigned k = 1; k < threads; k++)
            pool.emplace_back(parse_obj_range, buf.data(), cut[k], cut[k + 1], std::ref(parts[k]));
        parse_obj_range(buf.data(), cut[0], cut[1], parts[0]);
        for (auto& th : pool) th.join();
    }
    buf.clear();
    buf.shrink_to_fit();

    // every MTL file first, in file order (the reference's first pass, mesh.cpp:138-149, reads
    // them all before its second pass matches any usemtl line)
    std::vector<MtlEntry> mtls;
    for (const ObjPart& P : parts)
        for (const ObjPart::Event& e : P.events)
            if (e.kind == 0) {
                const int st = read_mtl(dir_of(path) + e.name, mtls);
                if (st != SPPM_OK) return st;
            }
    // then, in file order, the material switches and the first malformed face
    std::vector<int> mind;
    bool no_normals = false, no_texcoords = false, no_materials = true;
    int cmaterial = 0;
    std::vector<float> v, n, t;
    std::vector<int> vind, nind, tind;
    for (ObjPart& P : parts) {
        uint32_t done = 0;  // faces of this part given a material so far
        for (const ObjPart::Event& e : P.events) {
            mind.insert(mind.end(), e.face - done, cmaterial);
            done = e.face;
            if (e.kind == 0) {
                continue;
            } else if (e.kind == 1) {
                for (size_t i = 0; i < mtls.size(); i++) {
                    if (e.name == mtls[i].name) {
                        cmaterial = (int)i;
                        no_materials = false;
                        break;
                    }
                }
            } else {
                return fail(SPPM_ERR_IO, "'%s': face line with fewer than three vertices", path);
            }
        }
        mind.insert(mind.end(), P.faces - done, cmaterial);
        no_normals = no_normals || P.no_normals;
        no_texcoords = no_texcoords || P.no_texcoords;
        v.insert(v.end(), P.v.begin(), P.v.end());
        n.insert(n.end(), P.n.begin(), P.n.end());
        t.insert(t.end(), P.t.begin(), P.t.end());
        vind.insert(vind.end(), P.vind.begin(), P.vind.end());
        nind.insert(nind.end(), P.nind.begin(), P.nind.end());
        tind.insert(tind.end(), P.tind.begin(), P.tind.end());
        P = ObjPart();
    }

    std::unique_ptr<sppm_mesh> m(new sppm_mesh());
    const uint32_t nt = (uint32_t)mind.size();
    m->num_triangles = nt;
    m->positions.resize((size_t)nt * 9);
    m->normals.resize((size_t)nt * 9);
    m->texcoords.assign((size_t)nt * 6, 1.0e+30f);
    m->material_ids.assign(nt, 0);
    const size_t nv = v.size() / 3, nn = n.size() / 3;
    for (size_t k = 0; k < vind.size(); k++) {
        if (vind[k] < 0 || (size_t)vind[k] >= nv)
            return fail(SPPM_ERR_IO, "'%s': vertex index %d out of range", path, vind[k] + 1);
        if (!no_normals && (nind[k] < 0 || (size_t)nind[k] >= nn))
            return fail(SPPM_ERR_IO, "'%s': normal index %d out of range", path, nind[k] + 1);
        if (!no_texcoords && (tind[k] < 0 || (size_t)tind[k] >= t.size() / 2))
            return fail(SPPM_ERR_IO, "'%s': texture coordinate index %d out of range", path, tind[k] + 1);
    }
    for (uint32_t i = 0; i < nt; i++) {
        for (int k = 0; k < 3; k++) {
            const int vi = vind[i * 3 + k];
            for (int c = 0; c < 3; c++) m->positions[i * 9 + k * 3 + c] = v[vi * 3 + c] * scale + offset[c];
        }
    }
    for (uint32_t i = 0; i < nt; i++) {
        if (!no_normals) {
            for (int k = 0; k < 3; k++)
                for (int c = 0; c < 3; c++) m->normals[i * 9 + k * 3 + c] = n[nind[i * 3 + k] * 3 + c];
        } else {
            // face normal from the scaled positions (mesh.cpp:645-651)
            const V3 f = sppm::normalize3(sppm::cross3(m->pos(i, 1) - m->pos(i, 0), m->pos(i, 2) - m->pos(i, 0)));
            for (int k = 0; k < 3; k++) {
                m->normals[i * 9 + k * 3 + 0] = f.x;
                m->normals[i * 9 + k * 3 + 1] = f.y;
                m->normals[i * 9 + k * 3 + 2] = f.z;
            }
        }
    }

    bool have_light = false;
    if (!no_materials) {
        // material classification (mesh.cpp:520-611)
        for (size_t i = 0; i < mtls.size(); i++) {
            MtlEntry& e = mtls[i];
            int brdf = 0;
            float eta = 1.7f, specularity = 1.0f;
            const float ks2 = sppm::dot3(e.ks, e.ks);
            if (e.ns == 100.0f) {
                if (ks2 == 3.0f) brdf = 1;
                else if (ks2 > 0.0f) brdf = 3;
            } else {
                specularity = std::max(e.ns / 100.0f, 0.5f);
                if (ks2 == 3.0f) brdf = 4;
                else if (ks2 > 0.0f) brdf = 6;
            }
            if (e.name.compare(0, 5, "glass") == 0) {
                eta = ks2 / 3.0f + 1.0f;
                if (e.ns == 100.0f) brdf = 2;
                else {
                    specularity = std::max(e.ns / 100.0f, 0.5f);
                    brdf = 5;
                }
            }
            if (sppm::dot3(e.ka, e.ka) > 0.0f) {
                brdf = -1;
                have_light = true;
            }
            V3 kd = e.kd;
            if (brdf == 0 || brdf == 3) kd = kd * 0.9f;
            if (brdf == 2 || brdf == 5) kd = v3(sppm::sqrt_f32(kd.x), sppm::sqrt_f32(kd.y), sppm::sqrt_f32(kd.z));
            if (e.name.compare(0, 3, "sss") == 0)
                return fail(SPPM_ERR_UNSUPPORTED, "'%s': subsurface ('sss') materials are not supported", path);
            sppm_material mat;
            mat.color[0] = kd.x;
            mat.color[1] = kd.y;
            mat.color[2] = kd.z;
            mat.eta = eta;
            mat.brdf = brdf;
            mat.glossiness = packed_glossiness(specularity);
            m->materials.push_back(mat);
        }
        for (uint32_t i = 0; i < nt; i++) m->material_ids[i] = mind[i];
        // textures: each textured material's map_Kd resampled to a 512x512 layer
        // (gpurt.cpp:176-196); a triangle of a textured material keeps its texture coordinates
        // when every face vertex of the file has one (mesh.cpp:342-349, 657-666)
        m->material_texture.assign(mtls.size(), -1);
        const size_t layer_bytes = (size_t)SPPM_TEXTURE_RES * SPPM_TEXTURE_RES * 4;
        for (size_t i = 0; i < mtls.size(); i++) {
            if (!mtls[i].textured) continue;
            m->material_texture[i] = (int32_t)m->num_textures++;
            m->textures.resize(m->num_textures * layer_bytes);
            sppm_tex_resample(mtls[i].texture.data(), mtls[i].tex_w, mtls[i].tex_h,
                              m->textures.data() + (m->num_textures - 1) * layer_bytes);
        }
        if (!no_texcoords)
            for (uint32_t i = 0; i < nt; i++) {
                if (!mtls[mind[i]].textured) continue;
                for (int k = 0; k < 3; k++) {
                    m->texcoords[(size_t)i * 6 + k * 2] = t[(size_t)tind[i * 3 + k] * 2];
                    m->texcoords[(size_t)i * 6 + k * 2 + 1] = t[(size_t)tind[i * 3 + k] * 2 + 1];
                }
            }
    } else {
        // default material (mesh.cpp:615-620): brdf 0; its colour is never assigned in the
        // reference, so it keeps TVector3's zero default
        sppm_material mat;
        mat.color[0] = mat.color[1] = mat.color[2] = 0.0f;
        mat.eta = 0.0f;
        mat.brdf = 0;
        mat.glossiness = 0.0f;
        m->materials.push_back(mat);
        m->material_texture.assign(1, -1);
    }
    m->finish_geometry();
    if (have_light) m->prepare_lights();
    *out = m.release();
    return SPPM_OK;
}

extern "C" int sppm_mesh_from_arrays(uint32_t num_triangles, const float* positions, const float* normals,
                                     const int32_t* material_ids, uint32_t num_materials,
                                     const sppm_material* materials, sppm_mesh** out) {
    if (!out || (num_triangles && (!positions || !material_ids)) || !num_materials || !materials)
        return fail(SPPM_ERR_ARG, "sppm_mesh_from_arrays: null argument or no materials");
    *out = nullptr;
    std::unique_ptr<sppm_mesh> m(new sppm_mesh());
    m->num_triangles = num_triangles;
    m->positions.assign(positions, positions + (size_t)num_triangles * 9);
    m->normals.resize((size_t)num_triangles * 9);
    m->texcoords.assign((size_t)num_triangles * 6, 1.0e+30f);
    m->material_ids.assign(material_ids, material_ids + num_triangles);
    m->materials.assign(materials, materials + num_materials);
    for (uint32_t i = 0; i < num_triangles; i++) {
        if (material_ids[i] < 0 || (uint32_t)material_ids[i] >= num_materials)
            return fail(SPPM_ERR_ARG, "triangle %u: material id %d out of range", i, material_ids[i]);
        if (normals) {
            for (int k = 0; k < 9; k++) m->normals[(size_t)i * 9 + k] = normals[(size_t)i * 9 + k];
        } else {
            const V3 f = sppm::normalize3(sppm::cross3(m->pos(i, 1) - m->pos(i, 0), m->pos(i, 2) - m->pos(i, 0)));
            for (int k = 0; k < 3; k++) {
                m->normals[(size_t)i * 9 + k * 3 + 0] = f.x;
                m->normals[(size_t)i * 9 + k * 3 + 1] = f.y;
                m->normals[(size_t)i * 9 + k * 3 + 2] = f.z;
            }
        }
    }
    bool have_light = false;
    for (uint32_t i = 0; i < num_materials; i++) {
        if (materials[i].brdf < -1 || materials[i].brdf > 6)
            return fail(SPPM_ERR_ARG, "material %u: brdf %d not supported", i, materials[i].brdf);
        if (materials[i].brdf == -1) have_light = true;
    }
    m->finish_geometry();
    if (have_light) m->prepare_lights();
    *out = m.release();
    return SPPM_OK;
}

extern "C" int sppm_mesh_get_scene(const sppm_mesh* m, sppm_scene* s) {
    if (!m || !s) return fail(SPPM_ERR_ARG, "sppm_mesh_get_scene: null argument");
    memset(s, 0, sizeof(*s));
    s->num_triangles = m->num_triangles;
    s->positions = m->positions.data();
    s->normals = m->normals.data();
    s->texcoords = m->texcoords.data();
    s->material_ids = m->material_ids.data();
    s->num_materials = (uint32_t)m->materials.size();
    s->materials = m->materials.data();
    s->num_lights = (uint32_t)m->light_cdf.size();
    s->light_triangles = m->light_triangles.data();
    s->light_cdf = m->light_cdf.data();
    s->light_area = m->light_area;
    s->bbox_min[0] = m->bbox.mn.x;
    s->bbox_min[1] = m->bbox.mn.y;
    s->bbox_min[2] = m->bbox.mn.z;
    s->bbox_max[0] = m->bbox.mx.x;
    s->bbox_max[1] = m->bbox.mx.y;
    s->bbox_max[2] = m->bbox.mx.z;
    s->num_nodes = m->num_nodes;
    s->node_bounds = m->node_bounds.data();
    s->node_triangle = m->node_triangle.data();
    s->order_base = m->order_base.data();
    s->order_miss = m->order_miss.data();
    s->num_textures = m->num_textures;
    s->textures = m->num_textures ? m->textures.data() : nullptr;
    s->material_texture = m->material_texture.empty() ? nullptr : m->material_texture.data();
    return SPPM_OK;
}

extern "C" void sppm_mesh_destroy(sppm_mesh* m) { delete m; }
