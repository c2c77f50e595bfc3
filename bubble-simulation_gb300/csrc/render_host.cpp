// Host side of the headless visualisation: the orbit camera, the view
// uniform, the vis texture's lifetime, one frame of the renderer, the PNG
// writer and their extern "C" entry points (include/bubble_render.h).
#include <cuda_runtime_api.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/bubble_render.h"
#include "launch_render.h"
#include "physics.h"
#include "sim_handle.h"

namespace bubble {

namespace {

struct v3 {
    float x, y, z;
};
v3 add(v3 a, v3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
v3 scale(v3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
float dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
v3 cross(v3 a, v3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
float length(v3 a) { return std::sqrt(dot(a, a)); }
v3 normalize(v3 a) { return scale(a, 1.0f / length(a)); }
// Zero for a vector too short (or non-finite) to normalise.
v3 normalize_or_zero(v3 a) {
    const float rcp = 1.0f / length(a);
    if (std::isfinite(rcp) && rcp > 0.0f) return scale(a, rcp);
    return {0.0f, 0.0f, 0.0f};
}

// Pitch limit of the orbit camera, just short of the poles (src/camera.rs:34).
constexpr float kPitchLimit = 1.5533f;

v3 cam_offset(const bubble_camera &c) {
    const float sy = std::sin(c.yaw), cy = std::cos(c.yaw);
    const float sp = std::sin(c.pitch), cp = std::cos(c.pitch);
    return scale(v3{cp * sy, sp, cp * cy}, c.distance);
}
v3 cam_target(const bubble_camera &c) { return {c.target[0], c.target[1], c.target[2]}; }
v3 cam_eye(const bubble_camera &c) { return add(cam_target(c), cam_offset(c)); }
v3 cam_forward(const bubble_camera &c) { return scale(normalize(cam_offset(c)), -1.0f); }
v3 cam_right(const bubble_camera &c) { return normalize_or_zero(cross(cam_forward(c), v3{0.0f, 1.0f, 0.0f})); }
v3 cam_up(const bubble_camera &c) { return normalize_or_zero(cross(cam_right(c), cam_forward(c))); }

// 4x4 matrices, column-major: m[col * 4 + row].
using mat4 = std::array<float, 16>;

mat4 mul(const mat4 &a, const mat4 &b) {
    mat4 r{};
    for (int c = 0; c < 4; ++c)
        for (int i = 0; i < 4; ++i) {
            float s = 0.0f;
            for (int k = 0; k < 4; ++k) s += a[k * 4 + i] * b[c * 4 + k];
            r[c * 4 + i] = s;
        }
    return r;
}

// Right-handed perspective with depth in [0, 1] (the projection of
// src/camera.rs:65-66): x' = w x, y' = h y, z' = r z + r n, w' = -z.
mat4 perspective_rh(float fov_y, float aspect, float znear, float zfar) {
    const float h = std::cos(0.5f * fov_y) / std::sin(0.5f * fov_y);
    const float w = h / aspect;
    const float r = zfar / (znear - zfar);
    return mat4{w, 0, 0, 0, 0, h, 0, 0, 0, 0, r, -1, 0, 0, r * znear, 0};
}

// Right-handed view matrix looking from `eye` at `centre` with `up`.
mat4 look_at_rh(v3 eye, v3 centre, v3 up) {
    const v3 f = normalize(add(centre, scale(eye, -1.0f)));
    const v3 s = normalize(cross(f, up));
    const v3 u = cross(s, f);
    return mat4{s.x, u.x, -f.x, 0, s.y, u.y, -f.y, 0, s.z, u.z, -f.z, 0, -dot(eye, s), -dot(eye, u), dot(eye, f), 1};
}

// General inverse by cofactors, in double, rounded once to f32.
bool invert(const mat4 &mf, mat4 &out) {
    double m[16], inv[16];
    for (int k = 0; k < 16; ++k) m[k] = mf[k];
    inv[0] = m[5] * m[10] * m[15] - m[5] * m[11] * m[14] - m[9] * m[6] * m[15] + m[9] * m[7] * m[14] +
             m[13] * m[6] * m[11] - m[13] * m[7] * m[10];
    inv[4] = -m[4] * m[10] * m[15] + m[4] * m[11] * m[14] + m[8] * m[6] * m[15] - m[8] * m[7] * m[14] -
             m[12] * m[6] * m[11] + m[12] * m[7] * m[10];
    inv[8] = m[4] * m[9] * m[15] - m[4] * m[11] * m[13] - m[8] * m[5] * m[15] + m[8] * m[7] * m[13] +
             m[12] * m[5] * m[11] - m[12] * m[7] * m[9];
    inv[12] = -m[4] * m[9] * m[14] + m[4] * m[10] * m[13] + m[8] * m[5] * m[14] - m[8] * m[6] * m[13] -
              m[12] * m[5] * m[10] + m[12] * m[6] * m[9];
    inv[1] = -m[1] * m[10] * m[15] + m[1] * m[11] * m[14] + m[9] * m[2] * m[15] - m[9] * m[3] * m[14] -
             m[13] * m[2] * m[11] + m[13] * m[3] * m[10];
    inv[5] = m[0] * m[10] * m[15] - m[0] * m[11] * m[14] - m[8] * m[2] * m[15] + m[8] * m[3] * m[14] +
             m[12] * m[2] * m[11] - m[12] * m[3] * m[10];
    inv[9] = -m[0] * m[9] * m[15] + m[0] * m[11] * m[13] + m[8] * m[1] * m[15] - m[8] * m[3] * m[13] -
             m[12] * m[1] * m[11] + m[12] * m[3] * m[9];
    inv[13] = m[0] * m[9] * m[14] - m[0] * m[10] * m[13] - m[8] * m[1] * m[14] + m[8] * m[2] * m[13] +
              m[12] * m[1] * m[10] - m[12] * m[2] * m[9];
    inv[2] = m[1] * m[6] * m[15] - m[1] * m[7] * m[14] - m[5] * m[2] * m[15] + m[5] * m[3] * m[14] +
             m[13] * m[2] * m[7] - m[13] * m[3] * m[6];
    inv[6] = -m[0] * m[6] * m[15] + m[0] * m[7] * m[14] + m[4] * m[2] * m[15] - m[4] * m[3] * m[14] -
             m[12] * m[2] * m[7] + m[12] * m[3] * m[6];
    inv[10] = m[0] * m[5] * m[15] - m[0] * m[7] * m[13] - m[4] * m[1] * m[15] + m[4] * m[3] * m[13] +
              m[12] * m[1] * m[7] - m[12] * m[3] * m[5];
    inv[14] = -m[0] * m[5] * m[14] + m[0] * m[6] * m[13] + m[4] * m[1] * m[14] - m[4] * m[2] * m[13] -
              m[12] * m[1] * m[6] + m[12] * m[2] * m[5];
    inv[3] = -m[1] * m[6] * m[11] + m[1] * m[7] * m[10] + m[5] * m[2] * m[11] - m[5] * m[3] * m[10] -
             m[9] * m[2] * m[7] + m[9] * m[3] * m[6];
    inv[7] = m[0] * m[6] * m[11] - m[0] * m[7] * m[10] - m[4] * m[2] * m[11] + m[4] * m[3] * m[10] +
             m[8] * m[2] * m[7] - m[8] * m[3] * m[6];
    inv[11] = -m[0] * m[5] * m[11] + m[0] * m[7] * m[9] + m[4] * m[1] * m[11] - m[4] * m[3] * m[9] -
              m[8] * m[1] * m[7] + m[8] * m[3] * m[5];
    inv[15] = m[0] * m[5] * m[10] - m[0] * m[6] * m[9] - m[4] * m[1] * m[10] + m[4] * m[2] * m[9] +
              m[8] * m[1] * m[6] - m[8] * m[2] * m[5];
    const double det = m[0] * inv[0] + m[1] * inv[4] + m[2] * inv[8] + m[3] * inv[12];
    if (!(std::fabs(det) > 0.0) || !std::isfinite(det)) return false;
    for (int k = 0; k < 16; ++k) out[k] = (float)(inv[k] / det);
    return true;
}

mat4 view_proj(const bubble_camera &c, float aspect) {
    const mat4 proj = perspective_rh(c.fov_y, std::max(aspect, 1e-3f), c.znear, c.zfar);
    const mat4 view = look_at_rh(cam_eye(c), cam_target(c), v3{0.0f, 1.0f, 0.0f});
    return mul(proj, view);
}

// box_dimensions (src/gpu/render.rs:392-402)
void box_dimensions(const uint32_t grid[3], float half[3], float &cell) {
    const float n_max = (float)std::max({grid[0], grid[1], grid[2], 1u});
    for (int k = 0; k < 3; ++k) half[k] = 0.5f * (float)grid[k] / n_max;
    cell = 1.0f / n_max;
}

// FieldMode::default_gain / default_colormap (src/gpu/render.rs:46-65)
float default_gain(int mode) {
    switch (mode) {
        case BUBBLE_FIELD_PHI: return 0.5f;
        case BUBBLE_FIELD_SPEED: return 4.0f;
        case BUBBLE_FIELD_TEMPERATURE: return 15.0f;
        default: return 20.0f;
    }
}
int default_colormap(int mode) {
    switch (mode) {
        case BUBBLE_FIELD_PHI: return BUBBLE_COLORMAP_VIRIDIS;
        case BUBBLE_FIELD_TEMPERATURE: return BUBBLE_COLORMAP_SIGNED;
        default: return BUBBLE_COLORMAP_INFERNO;
    }
}

std::string check_settings(const bubble_render_settings &s) {
    if (s.field_mode < 0 || s.field_mode > 3) return "field_mode must be 0..3";
    if (s.colormap < 0 || s.colormap > 2) return "colormap must be 0..2";
    if (s.clip_axis < -1 || s.clip_axis > 2) return "clip_axis must be -1, 0, 1 or 2";
    const float vals[] = {s.iso_level, s.wall_opacity, s.samples_per_cell, s.exposure,
                          s.field_gain, s.absorption, s.background, s.clip_pos};
    for (float v : vals)
        if (!std::isfinite(v)) return "render settings must be finite";
    return {};
}

// ---- PNG (RGBA8, stored deflate blocks) -----------------------------------
uint32_t crc32_update(uint32_t crc, const uint8_t *p, size_t n) {
    static uint32_t table[256];
    static bool init = false;
    if (!init) {
        for (uint32_t i = 0; i < 256; ++i) {
            uint32_t c = i;
            for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            table[i] = c;
        }
        init = true;
    }
    for (size_t i = 0; i < n; ++i) crc = table[(crc ^ p[i]) & 0xFFu] ^ (crc >> 8);
    return crc;
}

void put_be32(std::vector<uint8_t> &v, uint32_t x) {
    v.push_back((uint8_t)(x >> 24));
    v.push_back((uint8_t)(x >> 16));
    v.push_back((uint8_t)(x >> 8));
    v.push_back((uint8_t)x);
}

void put_chunk(std::vector<uint8_t> &out, const char type[4], const std::vector<uint8_t> &data) {
    put_be32(out, (uint32_t)data.size());
    const size_t start = out.size();
    out.insert(out.end(), type, type + 4);
    out.insert(out.end(), data.begin(), data.end());
    const uint32_t crc = crc32_update(0xFFFFFFFFu, out.data() + start, out.size() - start) ^ 0xFFFFFFFFu;
    put_be32(out, crc);
}

}  // namespace

int write_png(const char *path, const uint8_t *rgba, uint32_t w, uint32_t h, std::string &err) {
    // raw scanlines: filter byte 0 + 4w bytes
    const size_t row = (size_t)w * 4 + 1;
    std::vector<uint8_t> raw(row * h);
    for (uint32_t y = 0; y < h; ++y) {
        raw[y * row] = 0;
        std::memcpy(&raw[y * row + 1], rgba + (size_t)y * w * 4, (size_t)w * 4);
    }
    // zlib stream: header, stored blocks of <= 65535 bytes, Adler-32
    std::vector<uint8_t> z;
    z.reserve(raw.size() + raw.size() / 65535 * 5 + 16);
    z.push_back(0x78);
    z.push_back(0x01);
    size_t pos = 0;
    do {
        const size_t n = std::min<size_t>(65535, raw.size() - pos);
        const bool last = pos + n == raw.size();
        z.push_back(last ? 1 : 0);
        z.push_back((uint8_t)(n & 0xFF));
        z.push_back((uint8_t)(n >> 8));
        z.push_back((uint8_t)(~n & 0xFF));
        z.push_back((uint8_t)((~n >> 8) & 0xFF));
        z.insert(z.end(), raw.begin() + (long)pos, raw.begin() + (long)(pos + n));
        pos += n;
    } while (pos < raw.size());
    uint32_t a = 1, b = 0;
    for (uint8_t c : raw) {
        a = (a + c) % 65521u;
        b = (b + a) % 65521u;
    }
    put_be32(z, (b << 16) | a);

    std::vector<uint8_t> png = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
    std::vector<uint8_t> ihdr;
    put_be32(ihdr, w);
    put_be32(ihdr, h);
    ihdr.push_back(8);  // bit depth
    ihdr.push_back(6);  // RGBA
    ihdr.push_back(0);
    ihdr.push_back(0);
    ihdr.push_back(0);
    put_chunk(png, "IHDR", ihdr);
    put_chunk(png, "IDAT", z);
    put_chunk(png, "IEND", {});
    FILE *f = std::fopen(path, "wb");
    if (!f) {
        err = std::string("cannot create ") + path;
        return BUBBLE_ERR_INVALID;
    }
    const size_t wrote = std::fwrite(png.data(), 1, png.size(), f);
    const int closed = std::fclose(f);
    if (wrote != png.size() || closed != 0) {
        err = std::string("failed to write ") + path;
        return BUBBLE_ERR_INVALID;
    }
    return BUBBLE_OK;
}

int make_view(const uint32_t grid[3], const bubble_render_settings &s, const bubble_camera *camera, uint32_t width,
              uint32_t height, uint32_t frame, bubble_view &v, std::string &err) {
    err = check_settings(s);
    if (!err.empty()) return BUBBLE_ERR_INVALID;
    if (width == 0 || height == 0 || width > 16384 || height > 16384) {
        err = "image size must be 1..16384 on each side";
        return BUBBLE_ERR_INVALID;
    }
    float half[3], cell;
    box_dimensions(grid, half, cell);
    bubble_camera cam;
    if (camera) {
        cam = *camera;
    } else {
        bubble_camera_default(&cam);
        bubble_camera_frame_box(&cam, half);
    }
    const mat4 vp = view_proj(cam, (float)width / (float)height);
    mat4 inv;
    if (!invert(vp, inv)) {
        err = "the camera's view-projection matrix is singular";
        return BUBBLE_ERR_INVALID;
    }
    std::memset(&v, 0, sizeof(v));
    std::memcpy(v.inv_view_proj, inv.data(), sizeof(v.inv_view_proj));
    const v3 eye = cam_eye(cam);
    v.cam_pos[0] = eye.x;
    v.cam_pos[1] = eye.y;
    v.cam_pos[2] = eye.z;
    for (int k = 0; k < 3; ++k) {
        v.box_half[k] = half[k];
        v.grid[k] = (float)grid[k];
    }
    v.box_half[3] = cell;
    v.render0[0] = s.iso_level;
    v.render0[1] = s.wall_opacity;
    v.render0[2] = s.samples_per_cell;
    v.render0[3] = s.exposure;
    v.render1[0] = (float)s.field_mode;
    v.render1[1] = (float)s.clip_axis;
    v.render1[2] = s.clip_pos;
    v.render1[3] = (float)s.colormap;
    v.render2[0] = s.field_gain;
    v.render2[1] = s.absorption;
    v.render2[2] = s.show_iso ? 1.0f : 0.0f;
    v.render2[3] = s.show_volume ? 1.0f : 0.0f;
    // the dither offset animates with the frame number (src/gpu/render.rs:312-314)
    v.render3[0] = (float)(frame % 64u) * 0.618034f;
    v.render3[1] = s.show_box ? 1.0f : 0.0f;
    v.render3[2] = s.background;
    return BUBBLE_OK;
}

#define VIS_CUDA(call, what)                                                   \
    do {                                                                       \
        const cudaError_t e_ = (call);                                         \
        if (e_ != cudaSuccess) {                                               \
            err = std::string(what) + ": " + cudaGetErrorString(e_);           \
            return BUBBLE_ERR_CUDA;                                            \
        }                                                                      \
    } while (0)

void Simulation::release_vis() {
    if (vis_tex_) cudaDestroyTextureObject(vis_tex_);
    if (vis_surf_) cudaDestroySurfaceObject(vis_surf_);
    if (vis_array_) cudaFreeArray(vis_array_);
    if (image_) cudaFree(image_);
    vis_tex_ = 0;
    vis_surf_ = 0;
    vis_array_ = nullptr;
    image_ = nullptr;
    image_bytes_ = 0;
    device_bytes_ -= std::min(device_bytes_, vis_bytes_);
    vis_bytes_ = 0;
}

int Simulation::visualise(std::string &err) {
    if (!state_) {
        err = "the simulation holds no lattice";
        return BUBBLE_ERR_INVALID;
    }
    if (!vis_array_) {
        int dev = 0, mx = 0, my = 0, mz = 0;
        VIS_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
        VIS_CUDA(cudaDeviceGetAttribute(&mx, cudaDevAttrMaxSurface3DWidth, dev), "cudaDeviceGetAttribute");
        VIS_CUDA(cudaDeviceGetAttribute(&my, cudaDevAttrMaxSurface3DHeight, dev), "cudaDeviceGetAttribute");
        VIS_CUDA(cudaDeviceGetAttribute(&mz, cudaDevAttrMaxSurface3DDepth, dev), "cudaDeviceGetAttribute");
        if (grid_[0] > (uint32_t)mx || grid_[1] > (uint32_t)my || grid_[2] > (uint32_t)mz) {
            err = "the lattice exceeds the largest 3-D surface of this device";
            return BUBBLE_ERR_INVALID;
        }
        const uint64_t bytes = n_cells_ * 8;
        size_t free_b = 0, total_b = 0;
        VIS_CUDA(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
        if ((double)bytes > 0.85 * (double)free_b) {
            err = "the visualisation texture needs " + std::to_string(bytes) + " bytes, above 85% of the " +
                  std::to_string(free_b) + " bytes free";
            return BUBBLE_ERR_MEMORY;
        }
        const cudaChannelFormatDesc desc = cudaCreateChannelDesc(16, 16, 16, 16, cudaChannelFormatKindFloat);
        cudaExtent ext;
        ext.width = grid_[0];
        ext.height = grid_[1];
        ext.depth = grid_[2];
        VIS_CUDA(cudaMalloc3DArray(&vis_array_, &desc, ext, cudaArraySurfaceLoadStore), "cudaMalloc3DArray");
        vis_bytes_ = bytes;
        device_bytes_ += bytes;
        cudaResourceDesc res;
        std::memset(&res, 0, sizeof(res));
        res.resType = cudaResourceTypeArray;
        res.res.array.array = vis_array_;
        VIS_CUDA(cudaCreateSurfaceObject(&vis_surf_, &res), "cudaCreateSurfaceObject");
        // the reference's sampler: clamp to edge, trilinear (src/gpu/render.rs:206-218)
        cudaTextureDesc td;
        std::memset(&td, 0, sizeof(td));
        td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeClamp;
        td.filterMode = cudaFilterModeLinear;
        td.readMode = cudaReadModeElementType;
        td.normalizedCoords = 1;
        VIS_CUDA(cudaCreateTextureObject(&vis_tex_, &res, &td, nullptr), "cudaCreateTextureObject");
    }
    const SimParamsHost h = sim_params(spec_.model, grid_);
    const float dof = spec_.eos == BUBBLE_EOS_BAG_DOF ? spec_.eos_param[0] : 1.0f;
    cudaError_t e;
    if (is_f64()) {
        e = launch::vis_f64((const V2<double> *)field_[cur_], (const V4<double> *)fluid_[cur_], params_f64(),
                            (double)h.a_rad, (double)h.t_ref, dof, vis_surf_, stream_);
    } else {
        e = launch::vis_f32((const V2<float> *)field_[cur_], (const V4<float> *)fluid_[cur_], params_f32(), h.a_rad,
                            h.t_ref, dof, arith_mode(), vis_surf_, stream_);
    }
    VIS_CUDA(e, "vis kernel");
    ++launches_;
    return BUBBLE_OK;
}

int Simulation::vis_copy(uint16_t *host, std::string &err) {
    if (!vis_array_) {
        err = "no visualisation texture yet: call bubble_visualise first";
        return BUBBLE_ERR_INVALID;
    }
    cudaMemcpy3DParms p;
    std::memset(&p, 0, sizeof(p));
    p.srcArray = vis_array_;
    p.dstPtr.ptr = host;
    p.dstPtr.pitch = (size_t)grid_[0] * 8;
    p.dstPtr.xsize = grid_[0];
    p.dstPtr.ysize = grid_[1];
    p.extent.width = grid_[0];
    p.extent.height = grid_[1];
    p.extent.depth = grid_[2];
    p.kind = cudaMemcpyDeviceToHost;
    VIS_CUDA(cudaMemcpy3DAsync(&p, stream_), "vis texture readback");
    VIS_CUDA(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    return BUBBLE_OK;
}

int Simulation::render(const bubble_view &view, uint32_t width, uint32_t height, uint8_t *host, std::string &err) {
    if (!vis_array_) {
        err = "no visualisation texture yet: call bubble_visualise first";
        return BUBBLE_ERR_INVALID;
    }
    const size_t bytes = (size_t)width * height * 4;
    if (bytes > image_bytes_) {
        if (image_) cudaFree(image_);
        image_ = nullptr;
        image_bytes_ = 0;
        VIS_CUDA(cudaMalloc(&image_, bytes), "cudaMalloc");
        image_bytes_ = bytes;
    }
    VIS_CUDA(launch::render(view, vis_tex_, (uchar4 *)image_, (int)width, (int)height, stream_), "render kernel");
    ++launches_;
    VIS_CUDA(cudaMemcpyAsync(host, image_, bytes, cudaMemcpyDeviceToHost, stream_), "image readback");
    VIS_CUDA(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    return BUBBLE_OK;
}

}  // namespace bubble

namespace {
int fail(int code, const std::string &msg) {
    bubble::set_last_error(msg);
    return code;
}
#define NEED(ptr)                                                     \
    do {                                                              \
        if (!(ptr)) return fail(BUBBLE_ERR_INVALID, #ptr " is NULL"); \
    } while (0)
}  // namespace

extern "C" {

int bubble_render_settings_default(bubble_render_settings *out) {
    NEED(out);
    out->field_mode = BUBBLE_FIELD_KINETIC;
    out->colormap = bubble::default_colormap(BUBBLE_FIELD_KINETIC);
    out->iso_level = 0.5f;
    out->wall_opacity = 0.55f;
    out->samples_per_cell = 1.5f;
    out->exposure = 1.5f;
    out->field_gain = bubble::default_gain(BUBBLE_FIELD_KINETIC);
    out->absorption = 12.0f;
    out->show_iso = 1;
    out->show_volume = 1;
    out->show_box = 1;
    out->background = 1.0f;
    out->clip_axis = -1;
    out->clip_pos = 0.0f;
    return BUBBLE_OK;
}

int bubble_render_settings_with_field(int32_t field_mode, bubble_render_settings *out) {
    NEED(out);
    if (field_mode < 0 || field_mode > 3) return fail(BUBBLE_ERR_INVALID, "field_mode must be 0..3");
    bubble_render_settings_default(out);
    out->field_mode = field_mode;
    out->colormap = bubble::default_colormap(field_mode);
    out->field_gain = bubble::default_gain(field_mode);
    return BUBBLE_OK;
}

int bubble_camera_default(bubble_camera *out) {
    NEED(out);
    out->target[0] = out->target[1] = out->target[2] = 0.0f;
    out->distance = 2.1f;
    out->yaw = 0.6f;
    out->pitch = 0.42f;
    out->fov_y = 50.0f * 3.14159265358979323846f / 180.0f;
    out->znear = 0.002f;
    out->zfar = 100.0f;
    return BUBBLE_OK;
}

int bubble_camera_frame_box(bubble_camera *c, const float half_extent[3]) {
    NEED(c);
    NEED(half_extent);
    c->target[0] = c->target[1] = c->target[2] = 0.0f;
    const float l = std::sqrt(half_extent[0] * half_extent[0] + half_extent[1] * half_extent[1] +
                              half_extent[2] * half_extent[2]);
    c->distance = l * 2.4f;
    return BUBBLE_OK;
}

int bubble_camera_orbit(bubble_camera *c, float dx, float dy) {
    NEED(c);
    c->yaw -= dx;
    c->pitch = std::min(std::max(c->pitch + dy, -bubble::kPitchLimit), bubble::kPitchLimit);
    return BUBBLE_OK;
}

int bubble_camera_pan(bubble_camera *c, float dx, float dy) {
    NEED(c);
    const float s = c->distance * 0.9f;
    const bubble::v3 r = bubble::cam_right(*c), u = bubble::cam_up(*c);
    const bubble::v3 d = bubble::add(bubble::scale(r, -dx * s), bubble::scale(u, dy * s));
    c->target[0] += d.x;
    c->target[1] += d.y;
    c->target[2] += d.z;
    return BUBBLE_OK;
}

int bubble_camera_zoom(bubble_camera *c, float amount) {
    NEED(c);
    c->distance = std::min(std::max(c->distance * (1.0f - amount * 0.12f), 0.02f), 40.0f);
    return BUBBLE_OK;
}

int bubble_camera_dolly(bubble_camera *c, float amount) {
    NEED(c);
    const bubble::v3 f = bubble::cam_forward(*c);
    const float k = amount * c->distance;
    c->target[0] += f.x * k;
    c->target[1] += f.y * k;
    c->target[2] += f.z * k;
    return BUBBLE_OK;
}

int bubble_camera_eye(const bubble_camera *c, float out[3]) {
    NEED(c);
    NEED(out);
    const bubble::v3 e = bubble::cam_eye(*c);
    out[0] = e.x;
    out[1] = e.y;
    out[2] = e.z;
    return BUBBLE_OK;
}

int bubble_camera_basis(const bubble_camera *c, float right[3], float up[3], float forward[3]) {
    NEED(c);
    const bubble::v3 r = bubble::cam_right(*c), u = bubble::cam_up(*c), f = bubble::cam_forward(*c);
    if (right) { right[0] = r.x; right[1] = r.y; right[2] = r.z; }
    if (up) { up[0] = u.x; up[1] = u.y; up[2] = u.z; }
    if (forward) { forward[0] = f.x; forward[1] = f.y; forward[2] = f.z; }
    return BUBBLE_OK;
}

int bubble_camera_view_proj(const bubble_camera *c, float aspect, float out[16]) {
    NEED(c);
    NEED(out);
    const bubble::mat4 m = bubble::view_proj(*c, aspect);
    std::memcpy(out, m.data(), sizeof(float) * 16);
    return BUBBLE_OK;
}

int bubble_render_box(const uint32_t grid[3], float half_extent[3], float *cell) {
    NEED(grid);
    NEED(half_extent);
    NEED(cell);
    bubble::box_dimensions(grid, half_extent, *cell);
    return BUBBLE_OK;
}

int bubble_render_view(const uint32_t grid[3], const bubble_render_settings *settings, const bubble_camera *camera,
                       uint32_t width, uint32_t height, uint32_t frame, bubble_view *out) {
    NEED(grid);
    NEED(settings);
    NEED(out);
    std::string err;
    const int rc = bubble::make_view(grid, *settings, camera, width, height, frame, *out, err);
    if (rc != BUBBLE_OK) return fail(rc, err);
    return BUBBLE_OK;
}

int bubble_visualise(bubble_sim *sim) {
    NEED(sim);
    std::string err;
    const int rc = sim->impl->visualise(err);
    if (rc != BUBBLE_OK) return fail(rc, err);
    return BUBBLE_OK;
}

int bubble_vis_copy(bubble_sim *sim, uint16_t *host) {
    NEED(sim);
    NEED(host);
    std::string err;
    const int rc = sim->impl->vis_copy(host, err);
    if (rc != BUBBLE_OK) return fail(rc, err);
    return BUBBLE_OK;
}

int bubble_render(bubble_sim *sim, const bubble_render_settings *settings, const bubble_camera *camera,
                  uint32_t width, uint32_t height, uint32_t frame, uint8_t *host) {
    NEED(sim);
    NEED(settings);
    NEED(host);
    std::string err;
    bubble_view v;
    int rc = bubble::make_view(sim->impl->grid(), *settings, camera, width, height, frame, v, err);
    if (rc == BUBBLE_OK) rc = sim->impl->render(v, width, height, host, err);
    if (rc != BUBBLE_OK) return fail(rc, err);
    return BUBBLE_OK;
}

int bubble_render_png(bubble_sim *sim, const bubble_render_settings *settings, uint32_t width, uint32_t height,
                      const char *path) {
    NEED(sim);
    NEED(settings);
    NEED(path);
    std::string err;
    bubble_view v;
    int rc = bubble::make_view(sim->impl->grid(), *settings, nullptr, width, height, 1, v, err);
    if (rc != BUBBLE_OK) return fail(rc, err);
    rc = sim->impl->visualise(err);
    if (rc != BUBBLE_OK) return fail(rc, err);
    std::vector<uint8_t> pixels((size_t)width * height * 4);
    rc = sim->impl->render(v, width, height, pixels.data(), err);
    if (rc == BUBBLE_OK) rc = bubble::write_png(path, pixels.data(), width, height, err);
    if (rc != BUBBLE_OK) return fail(rc, err);
    return BUBBLE_OK;
}

int bubble_write_png(const char *path, const uint8_t *rgba8, uint32_t width, uint32_t height) {
    NEED(path);
    NEED(rgba8);
    if (width == 0 || height == 0) return fail(BUBBLE_ERR_INVALID, "image size must be positive");
    std::string err;
    const int rc = bubble::write_png(path, rgba8, width, height, err);
    if (rc != BUBBLE_OK) return fail(rc, err);
    return BUBBLE_OK;
}

}  // extern "C"
