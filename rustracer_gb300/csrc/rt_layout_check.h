// Compile-time pins of the GPU struct layouts.  The sizes and offsets are the ones the reference's
// own tests pin: rustracer-renderer/tests/gpu_layout.rs:10-41 (struct spans equal the WGSL spans)
// and rustracer-core/src/material.rs:186-216 (MaterialGpu size/alignment/field offsets).
#pragma once
#include <cstddef>
#include "../../include/rustracer_cuda.h"

static_assert(sizeof(rt_bvh_node) == 48, "BVHNode is 48 bytes (bvh.rs:75-78)");
static_assert(offsetof(rt_bvh_node, left_first) == 12, "BVHNode.left_first");
static_assert(offsetof(rt_bvh_node, bbox_max) == 16, "BVHNode.bbox_max");
static_assert(offsetof(rt_bvh_node, right_child) == 28, "BVHNode.right_child");
static_assert(offsetof(rt_bvh_node, prim_count) == 32, "BVHNode.prim_count");

static_assert(sizeof(rt_triangle) == 128, "TriangleGpu is 128 bytes");
static_assert(offsetof(rt_triangle, v1) == 16 && offsetof(rt_triangle, v2) == 32, "TriangleGpu vertices");
static_assert(offsetof(rt_triangle, n0) == 48 && offsetof(rt_triangle, n2) == 80, "TriangleGpu normals");
static_assert(offsetof(rt_triangle, uv0) == 96 && offsetof(rt_triangle, uv2) == 112, "TriangleGpu uvs");
static_assert(offsetof(rt_triangle, material_id) == 120, "TriangleGpu.material_id");

static_assert(sizeof(rt_material) == 64 && alignof(rt_material) == 4, "MaterialGpu 64 B, align 4");
static_assert(offsetof(rt_material, emissive) == 16, "MaterialGpu.emissive");
static_assert(offsetof(rt_material, roughness) == 28, "MaterialGpu.roughness");
static_assert(offsetof(rt_material, metallic) == 32, "MaterialGpu.metallic");
static_assert(offsetof(rt_material, ior) == 36, "MaterialGpu.ior");
static_assert(offsetof(rt_material, kind) == 40, "MaterialGpu.kind");
static_assert(offsetof(rt_material, flags) == 44, "MaterialGpu.flags");
static_assert(offsetof(rt_material, tex_albedo) == 48, "MaterialGpu.tex_albedo");
static_assert(offsetof(rt_material, tex_mr) == 52, "MaterialGpu.tex_mr");
static_assert(offsetof(rt_material, tex_emissive) == 56, "MaterialGpu.tex_emissive");
static_assert(offsetof(rt_material, tex_normal) == 60, "MaterialGpu.tex_normal");

static_assert(sizeof(rt_light) == 64, "LightGpu is 64 bytes (scene.rs:128-140)");
static_assert(offsetof(rt_light, color) == 16 && offsetof(rt_light, intensity) == 28, "LightGpu colour");
static_assert(offsetof(rt_light, kind) == 32, "LightGpu.kind");

static_assert(sizeof(rt_camera_uniform) == 96, "CameraUniform is 96 bytes");
static_assert(offsetof(rt_camera_uniform, inv_half_res) == 64, "CameraUniform.inv_half_res");
static_assert(offsetof(rt_camera_uniform, focus_dist) == 84, "CameraUniform.focus_dist");

static_assert(sizeof(rt_photon) == 64, "PhotonGpu is 64 bytes");
static_assert(offsetof(rt_photon, power) == 16 && offsetof(rt_photon, incident) == 32, "PhotonGpu fields");

static_assert(sizeof(rt_image_params) == 80, "ImageParams is 80 bytes");
static_assert(offsetof(rt_image_params, light_emission) == 16, "ImageParams.light_emission");
static_assert(offsetof(rt_image_params, ambient) == 28, "ImageParams.ambient");
static_assert(offsetof(rt_image_params, photon_debug) == 52, "ImageParams.photon_debug");
static_assert(offsetof(rt_image_params, point_light_emission) == 56, "ImageParams.point_light_emission");
static_assert(offsetof(rt_image_params, _pad) == 68, "ImageParams._pad (debug view)");

static_assert(sizeof(rt_grid_params) == 48, "GridParamsUniform is 48 bytes");
static_assert(offsetof(rt_grid_params, grid_x) == 16 && offsetof(rt_grid_params, photon_slots) == 32, "GridParams");
static_assert(sizeof(rt_denoise_params) == 32, "DenoiseParamsUniform is 32 bytes");
static_assert(sizeof(rt_composite_params) == 16, "CompositeParams is 16 bytes");
static_assert(sizeof(rt_tonemap_params) == 32 && offsetof(rt_tonemap_params, marker) == 16, "ToneMapUniform");

// Backend-only structs (no reference counterpart): sizes the ctypes mirror relies on.
static_assert(sizeof(rt_render_config) == 96, "rt_render_config");
static_assert(sizeof(rt_camera) == 52, "rt_camera");
static_assert(sizeof(rt_wavefront_tuning) == 32, "rt_wavefront_tuning");
static_assert(sizeof(rt_server_config) == 64, "rt_server_config");
static_assert(sizeof(rt_request) == 164 && offsetof(rt_request, config) == 16 && offsetof(rt_request, camera) == 112,
              "rt_request");
static_assert(sizeof(rt_job_status) == 48, "rt_job_status");
static_assert(sizeof(rt_server_stats) == 128, "rt_server_stats");
static_assert(sizeof(rt_trace_profile) == 120 && offsetof(rt_trace_profile, record_bytes) == 112, "rt_trace_profile");
