// xr_path_tracer.hpp -- the reference's PathTracer render-pass interface in C++,
// on top of the C ABI of xr.h (header-only; link with libxr.so).
//
// Mirrors src/pathTracer.h:12-57 and src/pathTracer.cpp:35-201 for headless use:
//   PostTracerInit(scenes)     pathTracer.cpp:35-41   keeps the scene list, loads the current one
//   LoadCurrentScene(index)    pathTracer.cpp:162-167 upload + BVH build
//                              (ApplicationRT::CreateAccelerationStructures, ApplicationRT.cpp:55-66)
//   GetUniformBufferObject()   pathTracer.cpp:169-201 view / projection, their inverses, the
//                              previous frame's matrices, frame counter, bounces, toggles
//   DrawFrame()                pathTracer.cpp:57-81 / :135: frame counter modulo 10000, then Render
//   Render(ubo)                ApplicationReSTIRGI::Render (ApplicationReSTIRGI.cpp:150-275)
// UserSettings holds the fields of src/Editor/UserSettings.h:5-30 that the ReSTIR GI
// mode reads, plus the reuse parameters.  The camera is scripted (position, yaw,
// pitch) instead of the interactive fly camera.  Errors throw std::runtime_error
// with the library's message, as the reference's VK_CHECK throws (XVKCommon.h:10-16).
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "xr.h"

namespace xr {

inline void check(xr_status s, const XrContext* ctx = nullptr) {
    if (s != XR_OK) throw std::runtime_error(std::string("libxr: ") + xr_last_error(ctx));
}

// A scene in host memory in the reference's layouts (AVertex, u32 indices, AMaterial,
// per-model {index offset, vertex offset}) with its default camera.
struct HostScene {
    std::vector<XrVertex> vertices;
    std::vector<uint32_t> indices;
    std::vector<XrMaterial> materials;
    std::vector<XrMeshRange> ranges{XrMeshRange{0u, 0u}};
    XrCamera camera{};

    static HostScene Cornell() { return generate([](XrSceneData* d) { return xr_scene_cornell(d); }); }
    static HostScene Procedural(const XrProceduralDesc& desc) {
        return generate([&desc](XrSceneData* d) { return xr_scene_procedural(&desc, d); });
    }

  private:
    template <typename Fn>
    static HostScene generate(Fn fn) {
        XrSceneData d{};
        check(fn(&d));   // counts first (NULL arrays)
        HostScene s;
        s.vertices.resize(d.vertex_count);
        s.indices.resize(d.index_count);
        s.materials.resize(d.material_count);
        d.vertices = s.vertices.data();
        d.indices = s.indices.data();
        d.materials = s.materials.data();
        check(fn(&d));
        s.camera = d.camera;
        return s;
    }
};

struct UserSettings {
    uint32_t scene_index = 0;
    bool enable_sky_lighting = false;
    bool enable_reuse = true;
    uint32_t number_of_bounces = 4;
    float fov = 45.0f;
    bool compat_reference = false;   // the reference's own constants and quirks
    bool temporal_on = true;
    bool spatial_on = true;
    uint32_t m_cap_temporal = 20;
    uint32_t m_cap_spatial = 120;
    uint32_t n_neighbours = 5;
    float radius_px = 30.0f;
    bool visibility = true;
    uint32_t seed = 1;
};

class PathTracer {
  public:
    PathTracer(const UserSettings& settings, uint32_t width, uint32_t height, int device = 0)
        : settings_(settings), width_(width), height_(height) {
        XrDeviceDesc desc{device, width, height};
        check(xr_create(&desc, &ctx_));
        ApplySettings();
    }
    ~PathTracer() { xr_destroy(ctx_); }
    PathTracer(const PathTracer&) = delete;
    PathTracer& operator=(const PathTracer&) = delete;

    // pathTracer.cpp:35-41
    void PostTracerInit(std::vector<HostScene> scenes) {
        scenes_ = std::move(scenes);
        LoadCurrentScene(settings_.scene_index);
    }

    // pathTracer.cpp:162-167 + ApplicationRT.cpp:55-66
    void LoadCurrentScene(uint32_t index) {
        if (index >= scenes_.size()) throw std::out_of_range("PathTracer: no scene " + std::to_string(index));
        const HostScene& s = scenes_[index];
        check(xr_upload_scene(ctx_, s.vertices.data(), (uint32_t)s.vertices.size(), s.indices.data(),
                              (uint32_t)s.indices.size(), s.materials.data(), (uint32_t)s.materials.size(),
                              s.ranges.data(), (uint32_t)s.ranges.size()),
              ctx_);
        check(xr_build_bvh(ctx_), ctx_);
        camera_ = s.camera;
        camera_.fov_deg = settings_.fov;
        has_prev_ = false;
    }

    // pathTracer.cpp:169-201
    XrUniformBufferObject GetUniformBufferObject() {
        XrUniformBufferObject u{};
        check(xr_camera_ubo(&camera_, width_, height_, has_prev_ ? &prev_ : nullptr, current_frame_total_,
                            settings_.number_of_bounces, settings_.enable_sky_lighting ? 1u : 0u,
                            settings_.enable_reuse ? 1u : 0u, &u));
        prev_ = u;
        has_prev_ = true;
        return u;
    }

    // pathTracer.cpp:57-81 (frame counter modulo 10000, :135) + Render
    void DrawFrame() {
        current_frame_total_ = (current_frame_total_ + 1u) % 10000u;
        Render(GetUniformBufferObject());
    }

    // ApplicationReSTIRGI::Render: initial sample, temporal and spatial reuse, shading
    void Render(const XrUniformBufferObject& ubo) { check(xr_render_frame(ctx_, &ubo), ctx_); }

    // The tone-mapped RGBA8 image (XR_OUT_LDR8) or another output (waits for the frame).
    template <typename T>
    void ReadOutput(uint32_t which, std::vector<T>& out) {
        check(xr_read_output(ctx_, which, out.data(), out.size() * sizeof(T)), ctx_);
    }

    XrCamera& camera() { return camera_; }
    XrContext* context() { return ctx_; }
    uint32_t current_frame_total() const { return current_frame_total_; }

  private:
    void ApplySettings() {
        XrParams p;
        if (settings_.compat_reference) {
            xr_params_reference(&p, width_, height_);
        } else {
            xr_params_default(&p, width_, height_);
            p.temporal_on = settings_.temporal_on ? 1u : 0u;
            p.spatial_on = settings_.spatial_on ? 1u : 0u;
            p.m_cap_temporal = settings_.m_cap_temporal;
            p.m_cap_spatial = settings_.m_cap_spatial;
            p.n_neighbours = settings_.n_neighbours;
            p.radius_px = settings_.radius_px;
            p.visibility = settings_.visibility ? 1u : 0u;
            p.seed = settings_.seed;
        }
        check(xr_set_params(ctx_, &p), ctx_);
    }

    UserSettings settings_;
    uint32_t width_, height_;
    XrContext* ctx_ = nullptr;
    std::vector<HostScene> scenes_;
    XrCamera camera_{};
    XrUniformBufferObject prev_{};
    bool has_prev_ = false;
    uint32_t current_frame_total_ = 0;
};

}  // namespace xr
