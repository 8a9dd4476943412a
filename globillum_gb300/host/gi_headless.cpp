// gi_headless.cpp -- headless front-end over the C++ drop-in (gb_hybrid_pt.h),
// mirroring the progressive loop of the reference's `gi` binary
// (hl-main.cpp:617-711): register hybrid_pt, select it (activate), compute,
// then update while in_progress, and write the result image.
//
//   gi_headless <scene.bin> <out.pfm> [-r WxH] [-s spp] [-l path_length]
//               [--offsets ray shadow] [--halton] [--rr bounce]
//               [--algo hybrid_pt|gpu_area_lights|hybrid_area_lights] [--light-samples n]
//               (hybrid_area_lights: -s camera samples, --light-samples per camera sample)
//
// scene.bin (written by globillum_gb300.scenes.write_scene_bin): magic
// "GBSC", version 2 or 3, counts, then positions, normals, material indices,
// materials, principled parameters, lights and the camera; version 3 adds
// the diffuse textures, texture coordinates and per-material texture
// indices.  Little endian.
// The image is written like save_image (util.cpp:111-150): pixel (x, y) to
// (w-1-x, h-1-y), here as a float PFM.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "../../include/gb_hybrid_pt.h"

namespace {

struct SceneFile {
    std::vector<float> pos, nrm;
    std::vector<int> mat;
    std::vector<gb_material> mats;
    std::vector<gb_principled_params> params;
    std::vector<gb_light> lights;
    gb_camera cam{};
    // version 3: diffuse textures
    std::vector<std::vector<uint8_t>> pixels;
    std::vector<gb_texture> textures;
    std::vector<float> texcoords;  // 6 per triangle, empty without textures
    std::vector<int> dtex;         // per material, empty without textures
};

template <typename T> bool rd(std::ifstream& f, T* p, size_t n) {
    f.read(reinterpret_cast<char*>(p), (std::streamsize)(sizeof(T) * n));
    return (bool)f;
}

// Scene files carry rect lights only: a stored sky map pointer means nothing.
bool no_sky_maps(SceneFile* s) {
    for (gb_light& l : s->lights) {
        if (l.type == GB_LIGHT_SKY) return false;
        l.sky_rgb = nullptr;
    }
    return true;
}

bool load_scene(const char* path, SceneFile* s) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    char magic[4];
    int32_t hdr[5];  // version, triangles, materials, params, lights
    if (!rd(f, magic, 4) || std::memcmp(magic, "GBSC", 4) != 0 || !rd(f, hdr, 5) || (hdr[0] != 2 && hdr[0] != 3))
        return false;
    int nt = hdr[1], nm = hdr[2], np = hdr[3], nl = hdr[4];
    if (nt <= 0 || nm <= 0 || np < 0 || nl < 0) return false;
    s->pos.resize(9 * (size_t)nt);
    s->nrm.resize(9 * (size_t)nt);
    s->mat.resize(nt);
    s->mats.resize(nm);
    s->params.resize(np);
    s->lights.resize(nl);
    if (!(rd(f, s->pos.data(), s->pos.size()) && rd(f, s->nrm.data(), s->nrm.size()) &&
          rd(f, s->mat.data(), s->mat.size()) && rd(f, s->mats.data(), s->mats.size()) &&
          (np == 0 || rd(f, s->params.data(), s->params.size())) &&
          (nl == 0 || rd(f, s->lights.data(), s->lights.size())) && rd(f, &s->cam, 1) && no_sky_maps(s)))
        return false;
    if (hdr[0] == 2) return true;
    // version 3: int32 texture count, then per texture int32 w, h and w*h*4 bytes;
    // int32 flag, then (flag = 1) 6 floats per triangle and one int32 per material
    int32_t ntex = 0, flag = 0;
    if (!rd(f, &ntex, 1) || ntex < 0 || ntex > 4096) return false;
    s->pixels.resize(ntex);
    for (int k = 0; k < ntex; ++k) {
        int32_t wh[2];
        if (!rd(f, wh, 2) || wh[0] <= 0 || wh[1] <= 0 || (long long)wh[0] * wh[1] > (1ll << 26)) return false;
        s->pixels[k].resize(4 * (size_t)wh[0] * wh[1]);
        if (!rd(f, s->pixels[k].data(), s->pixels[k].size())) return false;
        s->textures.push_back(gb_texture{wh[0], wh[1], s->pixels[k].data()});
    }
    if (!rd(f, &flag, 1)) return false;
    if (flag == 1) {
        s->texcoords.resize(6 * (size_t)nt);
        s->dtex.resize(nm);
        if (!rd(f, s->texcoords.data(), s->texcoords.size()) || !rd(f, s->dtex.data(), s->dtex.size())) return false;
    }
    return true;
}

bool write_pfm(const char* path, int w, int h, const std::vector<float>& rgb) {
    std::FILE* f = std::fopen(path, "wb");
    if (!f) return false;
    std::fprintf(f, "PF\n%d %d\n-1.0\n", w, h);
    // PFM stores rows bottom to top; save_image mirrors x and y
    std::vector<float> row(3 * (size_t)w);
    for (int r = 0; r < h; ++r) {
        int y = r;  // PFM row r (from the bottom) = image row h-1-r from the top = source row r after the y flip
        for (int x = 0; x < w; ++x)
            for (int k = 0; k < 3; ++k) row[3 * (size_t)x + k] = rgb[3 * ((size_t)y * w + (w - 1 - x)) + k];
        std::fwrite(row.data(), sizeof(float), row.size(), f);
    }
    std::fclose(f);
    return true;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 3) {
        std::fprintf(stderr,
                     "usage: %s scene.bin out.pfm [-r WxH] [-s spp] [-l len] [--offsets r s] [--halton] [--rr b]"
                     " [--algo hybrid_pt|gpu_area_lights|hybrid_area_lights] [--light-samples n]\n",
                     argv[0]);
        return 2;
    }
    int w = 256, h = 256, spp = gb::init_path_samples(), len = gb::init_path_length(), rr = -1;
    float ro = 0.3f, so = 0.9f;
    bool halton = false;
    std::string algo_name = "hybrid_pt";
    int light_samples = 32;
    for (int i = 3; i < argc; ++i) {
        std::string a = argv[i];
        if (a == "-r" && i + 1 < argc) std::sscanf(argv[++i], "%dx%d", &w, &h);
        else if (a == "-s" && i + 1 < argc) spp = std::atoi(argv[++i]);
        else if (a == "-l" && i + 1 < argc) len = std::atoi(argv[++i]);
        else if (a == "--offsets" && i + 2 < argc) { ro = (float)std::atof(argv[++i]); so = (float)std::atof(argv[++i]); }
        else if (a == "--halton") halton = true;
        else if (a == "--rr" && i + 1 < argc) rr = std::atoi(argv[++i]);
        else if (a == "--algo" && i + 1 < argc) algo_name = argv[++i];
        else if (a == "--light-samples" && i + 1 < argc) light_samples = std::atoi(argv[++i]);
        else { std::fprintf(stderr, "unknown argument %s\n", a.c_str()); return 2; }
    }
    SceneFile sf;
    if (!load_scene(argv[1], &sf)) { std::fprintf(stderr, "cannot read scene %s\n", argv[1]); return 1; }
    gb_scene_desc sd{};
    sd.num_triangles = (int)sf.mat.size();
    sd.positions = sf.pos.data();
    sd.normals = sf.nrm.data();
    sd.material_index = sf.mat.data();
    sd.num_materials = (int)sf.mats.size();
    sd.materials = sf.mats.data();
    sd.num_params = (int)sf.params.size();
    sd.params = sf.params.empty() ? nullptr : sf.params.data();
    sd.num_lights = (int)sf.lights.size();
    sd.lights = sf.lights.empty() ? nullptr : sf.lights.data();
    sd.num_textures = (int)sf.textures.size();
    sd.textures = sf.textures.empty() ? nullptr : sf.textures.data();
    sd.texcoords = sf.texcoords.empty() ? nullptr : sf.texcoords.data();
    sd.diffuse_texture = sf.dtex.empty() ? nullptr : sf.dtex.data();
    gb::rt_set set;
    set.scene = &sd;
    set.camera = sf.cam;
    set.w = w; set.h = h;
    try {
        gb::init_path_samples() = spp;
        gb::init_path_length() = len;
        // the algorithms register, one is selected (hl-main.cpp:612-628)
        gb::hybrid_pt algo(w, h);
        gb::gpu_area_lights direct(w, h);
        gb::hybrid_area_lights hybrid_direct(w, h);
        hybrid_direct.render_desc().shadow_offset = so;
        algo.render_desc().ray_offset = ro;
        algo.render_desc().shadow_offset = so;
        algo.render_desc().rng_mode = halton ? GB_RNG_HALTON_LIGHT : GB_RNG_MRG32K3A_POOL;
        algo.render_desc().rr_start = rr;
        gb::gi_algorithm::original_rt_set() = &set;
        gb::gi_algorithm::select(algo_name);
        gb::gi_algorithm* a = gb::gi_algorithm::selected();
        if (a == &direct || a == &hybrid_direct) a->light_samples(light_samples);
        if (a == &hybrid_direct) a->path_samples(spp);
        a->compute();
        while (a->in_progress()) a->update();
        std::vector<float> img = a == &algo ? algo.result() : a == &direct ? direct.result() : hybrid_direct.result();
        if (!write_pfm(argv[2], w, h, img)) { std::fprintf(stderr, "cannot write %s\n", argv[2]); return 1; }
        if (a == &algo)
            std::printf("rendered %dx%d, %d paths of length %d per pixel\n", w, h, algo.paths_done(), len);
        else if (a == &direct)
            std::printf("rendered %dx%d, %d direct light samples per pixel\n", w, h, light_samples);
        else
            std::printf("rendered %dx%d, %d camera x %d light samples per pixel\n", w, h, spp, light_samples);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
