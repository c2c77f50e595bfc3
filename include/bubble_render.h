/*
 * Headless visualisation: the vis pack and the volume ray-march, as CUDA
 * kernels writing a device image, plus the offscreen PNG capture.
 *
 * Replaces, for a machine without a graphics API:
 *   - `Simulation::record_visualisation` (src/gpu/sim.rs:918-942) and the
 *     vis pass (shaders/vis.wgsl:30-55): the packed rgba16float 3-D texture
 *     of (phi/phi_b, |v|, T/T_ref - 1, (E+p)v^2/e_ref);
 *   - `VolumeRenderer` (src/gpu/render.rs:140-390) and its fragment shader
 *     (shaders/volume.wgsl:229-381): one ray per pixel through that texture;
 *   - `capture::render_to_png` (src/capture.rs:19-117);
 *   - `OrbitCamera` (src/camera.rs:9-105) and `RenderSettings`
 *     (src/gpu/render.rs:69-128).
 *
 * The texture is a CUDA array of half4 written through a surface by the vis
 * kernel and sampled with hardware trilinear filtering (clamp to edge,
 * normalised coordinates), as the reference's sampler does
 * (src/gpu/render.rs:206-218).  It is allocated on the first
 * bubble_visualise call (8 B per cell) and released by bubble_resize and
 * bubble_destroy.
 */
#ifndef BUBBLE_RENDER_H
#define BUBBLE_RENDER_H

#include <stddef.h>
#include <stdint.h>

#include "bubble.h"

#ifdef __cplusplus
extern "C" {
#endif

/* FieldMode (src/gpu/render.rs:17-28). */
#define BUBBLE_FIELD_PHI 0
#define BUBBLE_FIELD_SPEED 1
#define BUBBLE_FIELD_TEMPERATURE 2
#define BUBBLE_FIELD_KINETIC 3

/* COLORMAPS (src/gpu/render.rs:67): viridis, inferno, signed. */
#define BUBBLE_COLORMAP_VIRIDIS 0
#define BUBBLE_COLORMAP_INFERNO 1
#define BUBBLE_COLORMAP_SIGNED 2

/* RenderSettings (src/gpu/render.rs:69-94). */
typedef struct bubble_render_settings {
    int32_t field_mode;
    int32_t colormap;
    float iso_level;
    float wall_opacity;
    float samples_per_cell;
    float exposure;
    float field_gain;
    float absorption;
    int32_t show_iso;
    int32_t show_volume;
    int32_t show_box;
    float background;
    int32_t clip_axis; /* -1 off, 0/1/2 = x/y/z half-space */
    float clip_pos;    /* in [-1, 1] along the clip axis */
} bubble_render_settings;

/* OrbitCamera (src/camera.rs:9-32). */
typedef struct bubble_camera {
    float target[3];
    float distance;
    float yaw;
    float pitch;
    float fov_y;
    float znear;
    float zfar;
} bubble_camera;

/* The 176-byte `ViewUniform` (src/gpu/render.rs:130-139,
 * shaders/volume.wgsl:22-31), column-major inv_view_proj then seven vec4s. */
typedef struct bubble_view {
    float inv_view_proj[16];
    float cam_pos[4];
    float box_half[4]; /* xyz half extents (longest axis spans 1), w = cell */
    float grid[4];
    float render0[4]; /* iso_level, wall_opacity, samples_per_cell, exposure */
    float render1[4]; /* field_mode, clip_axis, clip_pos, colormap */
    float render2[4]; /* field_gain, absorption, show_iso, show_volume */
    float render3[4]; /* frame_jitter, show_box, background, 0 */
} bubble_view;

/* RenderSettings::default (src/gpu/render.rs:110-128). */
int bubble_render_settings_default(bubble_render_settings *out);
/* RenderSettings::with_field (src/gpu/render.rs:96-107): the field's
 * default gain and colour map (src/gpu/render.rs:46-65). */
int bubble_render_settings_with_field(int32_t field_mode, bubble_render_settings *out);

/* OrbitCamera::default (src/camera.rs:21-32). */
int bubble_camera_default(bubble_camera *out);
/* OrbitCamera::frame_box (src/camera.rs:101-104). */
int bubble_camera_frame_box(bubble_camera *c, const float half_extent[3]);
/* OrbitCamera::orbit / pan / zoom / dolly (src/camera.rs:73-99). */
int bubble_camera_orbit(bubble_camera *c, float dx, float dy);
int bubble_camera_pan(bubble_camera *c, float dx, float dy);
int bubble_camera_zoom(bubble_camera *c, float amount);
int bubble_camera_dolly(bubble_camera *c, float amount);
/* OrbitCamera::eye / right / up (src/camera.rs:36-62). */
int bubble_camera_eye(const bubble_camera *c, float out[3]);
int bubble_camera_basis(const bubble_camera *c, float right[3], float up[3], float forward[3]);
/* OrbitCamera::view_proj (src/camera.rs:64-69), column-major. */
int bubble_camera_view_proj(const bubble_camera *c, float aspect, float out[16]);

/* box_dimensions (src/gpu/render.rs:392-402): half extents normalised so
 * the longest axis spans 1, and the world size of one cell. */
int bubble_render_box(const uint32_t grid[3], float half_extent[3], float *cell);

/* VolumeRenderer::update (src/gpu/render.rs:268-322): the uniform of frame
 * number `frame` (1 for the first frame after creation).  `camera` NULL
 * means the default camera framed on the box, as render_to_png does
 * (src/capture.rs:46-48). */
int bubble_render_view(const uint32_t grid[3], const bubble_render_settings *settings,
                       const bubble_camera *camera, uint32_t width, uint32_t height,
                       uint32_t frame, bubble_view *out);

/* Simulation::record_visualisation (src/gpu/sim.rs:918-942): recover the
 * primitives of the current slot and write the vis texture. */
int bubble_visualise(bubble_sim *sim);

/* Copies the vis texture to host memory as nx*ny*nz half4 texels (raw
 * IEEE binary16 bits, x fastest), for inspection and tests. */
int bubble_vis_copy(bubble_sim *sim, uint16_t *host_rgba16);

/* One frame of the volume renderer over the current vis texture (call
 * bubble_visualise first): width*height RGBA8 pixels, row 0 at the top, into
 * host memory.  `camera` NULL = default camera framed on the box; `frame`
 * as in bubble_render_view. */
int bubble_render(bubble_sim *sim, const bubble_render_settings *settings,
                  const bubble_camera *camera, uint32_t width, uint32_t height,
                  uint32_t frame, uint8_t *host_rgba8);

/* capture::render_to_png (src/capture.rs:19-117): refreshes the vis
 * texture, renders one frame (default framed camera, frame 1) and writes an
 * RGBA8 PNG. */
int bubble_render_png(bubble_sim *sim, const bubble_render_settings *settings,
                      uint32_t width, uint32_t height, const char *path);

/* Writes width*height RGBA8 pixels as a PNG (stored deflate blocks). */
int bubble_write_png(const char *path, const uint8_t *rgba8, uint32_t width, uint32_t height);

#ifdef __cplusplus
}
#endif

#endif /* BUBBLE_RENDER_H */
