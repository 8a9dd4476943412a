// gb_hybrid_pt.h -- C++ drop-in for globillum's integrator plugin API on top
// of the C ABI (gbpt.h).  Header-only; link libgbpt.so.
//
// gi_algorithm mirrors the reference's plugin base class (gi_algorithm.h:12-68):
// a name-keyed registry (duplicate names throw std::logic_error, unknown
// names std::runtime_error), activate-once semantics, compute/update/
// progressive/in_progress and the path_samples / path_length /
// light_samples knobs with the same default messages.  Its rta::rt_set
// argument becomes gb::rt_set (scene description + camera + resolution).
//
// hybrid_pt replaces the reference's hybrid_pt (hybrid-pt.h:256-288,
// hybrid-pt.cpp:65-174): activate uploads the scene and builds the BVH,
// compute starts a progressive pass, every update renders one further path
// sample of every pixel on the GPU (the reference's update advances one
// trace + bounce), in_progress reports whether path samples remain, and
// result() returns output_color.
#pragma once

#include <iostream>
#include <list>
#include <stdexcept>
#include <string>
#include <vector>

#include "gbpt.h"

namespace gb {

// Stand-in for rta::rt_set: what activate() needs to set up the path.
struct rt_set {
    const gb_scene_desc* scene = nullptr;
    gb_camera camera{};
    int w = 0, h = 0;
    int device = 0;
};

inline int& init_path_samples() { static int v = 2; return v; }  // gi_algorithm.cpp:3
inline int& init_path_length() { static int v = 2; return v; }
inline int& init_light_samples() { static int v = 2; return v; }

class gi_algorithm {
public:
    static rt_set*& original_rt_set() { static rt_set* s = nullptr; return s; }
    static gi_algorithm*& selected() { static gi_algorithm* s = nullptr; return s; }

protected:
    static std::vector<gi_algorithm*>& algorithms() { static std::vector<gi_algorithm*> a; return a; }
    bool activated;
    std::string name;
    bool verbose;

public:
    explicit gi_algorithm(const std::string& name) : activated(false), name(name), verbose(false) {
        for (auto* a : algorithms())
            if (a->name == name) throw std::logic_error(std::string("the algorithm ") + name + " is already registered.");
        algorithms().push_back(this);
    }
    virtual ~gi_algorithm() {
        auto& a = algorithms();
        for (size_t i = 0; i < a.size(); ++i)
            if (a[i] == this) { a.erase(a.begin() + (long)i); break; }
        if (selected() == this) selected() = nullptr;
    }
    virtual void activate(rt_set* /*orig_set*/) { activated = true; }
    virtual void compute() = 0;
    virtual bool progressive() { return false; }
    virtual bool in_progress() { return false; }
    virtual void update() { compute(); }

    static void select(const std::string& name) {
        for (auto* a : algorithms())
            if (a->name == name) {
                selected() = a;
                if (!a->activated) a->activate(original_rt_set());
                return;
            }
        throw std::runtime_error("no gi algorithm called " + name);
    }
    static gi_algorithm* get(const std::string& name) {
        for (auto* a : algorithms())
            if (a->name == name) return a;
        return nullptr;
    }
    static std::list<std::string> list() {
        std::list<std::string> l;
        for (auto* a : algorithms()) l.push_back(a->name);
        return l;
    }
    void debug(bool verb) { verbose = verb; }
    const std::string& algorithm_name() const { return name; }

    virtual void path_samples(int) { std::cerr << "the algorithm '" << name << "' does not know about path samples." << std::endl; }
    virtual void path_length(int) { std::cerr << "the algorithm '" << name << "' does not know about path length." << std::endl; }
    virtual void light_samples(int) { std::cerr << "the algorithm '" << name << "' does not know about light samples." << std::endl; }
};

// Throws std::runtime_error carrying gb_last_error for a failing call.
inline void gb_check(gb_ctx* ctx, int rc, const char* what) {
    if (rc != GB_OK)
        throw std::runtime_error(std::string(what) + " failed (" + std::to_string(rc) + "): " +
                                 (ctx ? gb_last_error(ctx) : "no context"));
}

class hybrid_pt : public gi_algorithm {
protected:
    int w, h;
    gb_ctx* ctx = nullptr;
    gb_scene* scene = nullptr;
    gb_camera cam{};
    gb_render_desc desc{};
    int spp, len;
    bool pass_started = false;

public:
    hybrid_pt(int w, int h, const std::string& name = "hybrid_pt")
        : gi_algorithm(name), w(w), h(h), spp(init_path_samples()), len(init_path_length()) {
        // reference parameters: curand seed 0, offsets 0.3 / 0.9, white
        // background, no Russian roulette
        desc.width = w; desc.height = h;
        desc.rng_mode = GB_RNG_MRG32K3A_POOL;
        desc.seed = 0;
        desc.ray_offset = 0.3f;
        desc.shadow_offset = 0.9f;
        desc.background[0] = desc.background[1] = desc.background[2] = 1.0f;
        desc.rr_start = -1;
    }
    ~hybrid_pt() override {
        if (scene) gb_scene_destroy(scene);
        if (ctx) gb_ctx_destroy(ctx);
    }
    void activate(rt_set* set) override {
        if (activated) return;
        if (!set || !set->scene) throw std::runtime_error("hybrid_pt::activate: no scene");
        gi_algorithm::activate(set);
        gb_ctx_desc cd{set->device, nullptr};
        int rc = gb_ctx_create(&cd, &ctx);
        if (rc != GB_OK) throw std::runtime_error("gb_ctx_create failed (" + std::to_string(rc) + ")");
        gb_check(ctx, gb_scene_create(ctx, set->scene, &scene), "gb_scene_create");
        cam = set->camera;
    }
    void set_camera(const gb_camera& c) { cam = c; }
    // render parameters beyond the reference's fixed ones (offsets for
    // other scene scales, Halton light samples, Russian roulette)
    gb_render_desc& render_desc() { return desc; }
    void compute() override {
        if (!activated) throw std::runtime_error("hybrid_pt::compute before activate");
        desc.width = w; desc.height = h;
        desc.spp = spp;
        desc.max_bounces = len;
        gb_check(ctx, gb_render_begin(ctx, scene, &cam, &desc), "gb_render_begin");
        pass_started = true;
        update();
    }
    void update() override {
        if (!pass_started) { compute(); return; }
        if (in_progress()) gb_check(ctx, gb_render_step(ctx, 1), "gb_render_step");
    }
    bool progressive() override { return true; }
    bool in_progress() override {
        if (!pass_started) return false;
        int done = 0;
        gb_render_paths_done(ctx, &done);
        return done < spp;
    }
    int paths_done() const {
        int done = 0;
        if (ctx) gb_render_paths_done(ctx, &done);
        return done;
    }
    void path_samples(int n) override { spp = n; }
    void path_length(int n) override { len = n; }
    // output_color (hybrid-pt.h:35): w*h*3 floats, pixel (x,y) at y*w+x.
    std::vector<float> result() {
        std::vector<float> out((size_t)w * h * 3);
        gb_check(ctx, gb_render_read(ctx, out.data(), 0), "gb_render_read");
        return out;
    }
};

// gpu_area_lights (direct-lighting.cpp:29-104, registered under that name):
// compute renders the first-hit material colour times the average of
// light_samples area-light samples (32 by default, as the reference's
// evaluator is constructed) in one call; update is a no-op once done.
class gpu_area_lights : public gi_algorithm {
protected:
    int w, h;
    gb_ctx* ctx = nullptr;
    gb_scene* scene = nullptr;
    gb_camera cam{};
    gb_render_desc desc{};
    int samples = 32;
    std::vector<float> image;

public:
    gpu_area_lights(int w, int h, const std::string& name = "gpu_area_lights") : gi_algorithm(name), w(w), h(h) {
        desc.width = w; desc.height = h;
        desc.spp = 1; desc.max_bounces = 1;
        desc.rng_mode = GB_RNG_MRG32K3A_POOL;
        desc.seed = 0;
        desc.shadow_offset = 0.01f;  // the GPU sampler's offset (arealight-sampler.cu:230)
        desc.background[0] = desc.background[1] = desc.background[2] = 1.0f;
        desc.rr_start = -1;
    }
    ~gpu_area_lights() override {
        if (scene) gb_scene_destroy(scene);
        if (ctx) gb_ctx_destroy(ctx);
    }
    void activate(rt_set* set) override {
        if (activated) return;
        if (!set || !set->scene) throw std::runtime_error("gpu_area_lights::activate: no scene");
        gi_algorithm::activate(set);
        gb_ctx_desc cd{set->device, nullptr};
        int rc = gb_ctx_create(&cd, &ctx);
        if (rc != GB_OK) throw std::runtime_error("gb_ctx_create failed (" + std::to_string(rc) + ")");
        gb_check(ctx, gb_scene_create(ctx, set->scene, &scene), "gb_scene_create");
        cam = set->camera;
    }
    void set_camera(const gb_camera& c) { cam = c; }
    gb_render_desc& render_desc() { return desc; }
    void compute() override {
        if (!activated) throw std::runtime_error("gpu_area_lights::compute before activate");
        desc.width = w; desc.height = h;
        image.assign((size_t)w * h * 3, 0.0f);
        gb_check(ctx, gb_render_direct(ctx, scene, &cam, &desc, samples, image.data(), 0), "gb_render_direct");
    }
    void update() override {}
    bool progressive() override { return true; }
    bool in_progress() override { return false; }
    void light_samples(int n) override { samples = n; }
    std::vector<float> result() const { return image; }
};

// hybrid_area_lights (direct-lighting.cpp:203-316): `path_samples` jittered
// camera samples per pixel, each with `light_samples` samples of the CPU
// area-light sampler, over gb_render_hybrid_direct.  The reference's
// constructor hands init_light_samples to the camera-sample count and
// init_path_samples to the per-camera light-sample count
// (direct-lighting.cpp:222-226 against direct-lighting.h:152-157); the
// knobs then set each count by its own name.  Both start at 2.
class hybrid_area_lights : public gi_algorithm {
protected:
    int w, h;
    gb_ctx* ctx = nullptr;
    gb_scene* scene = nullptr;
    gb_camera cam{};
    gb_render_desc desc{};
    int cam_samples = 2, samples_per_cam = 2;
    std::vector<float> image;

public:
    hybrid_area_lights(int w, int h, const std::string& name = "hybrid_area_lights")
        : gi_algorithm(name), w(w), h(h) {
        desc.width = w; desc.height = h;
        desc.spp = 1; desc.max_bounces = 1;
        desc.rng_mode = GB_RNG_MRG32K3A_POOL;
        desc.seed = 0;
        desc.shadow_offset = 0.9f;  // the CPU sampler's offset (arealight-sampler-cpu.cpp:115)
        desc.background[0] = desc.background[1] = desc.background[2] = 1.0f;
        desc.rr_start = -1;
    }
    ~hybrid_area_lights() override {
        if (scene) gb_scene_destroy(scene);
        if (ctx) gb_ctx_destroy(ctx);
    }
    void activate(rt_set* set) override {
        if (activated) return;
        if (!set || !set->scene) throw std::runtime_error("hybrid_area_lights::activate: no scene");
        gi_algorithm::activate(set);
        gb_ctx_desc cd{set->device, nullptr};
        int rc = gb_ctx_create(&cd, &ctx);
        if (rc != GB_OK) throw std::runtime_error("gb_ctx_create failed (" + std::to_string(rc) + ")");
        gb_check(ctx, gb_scene_create(ctx, set->scene, &scene), "gb_scene_create");
        cam = set->camera;
    }
    void set_camera(const gb_camera& c) { cam = c; }
    gb_render_desc& render_desc() { return desc; }
    void compute() override {
        if (!activated) throw std::runtime_error("hybrid_area_lights::compute before activate");
        desc.width = w; desc.height = h;
        image.assign((size_t)w * h * 3, 0.0f);
        gb_check(ctx, gb_render_hybrid_direct(ctx, scene, &cam, &desc, cam_samples, samples_per_cam, image.data(), 0),
                 "gb_render_hybrid_direct");
    }
    void update() override {}
    bool progressive() override { return true; }
    bool in_progress() override { return false; }
    void light_samples(int n) override { samples_per_cam = n; }
    void path_samples(int n) override { cam_samples = n; }
    std::vector<float> result() const { return image; }
};

}  // namespace gb
