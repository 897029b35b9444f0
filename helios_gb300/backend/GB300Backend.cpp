/** GB300Backend.cpp -- helios::RayTracingBackend over the libhrt C ABI.
 *
 * Semantics follow the reference backend each virtual replaces
 * (plugins/radiation/src/backends/OptiX8Backend.cpp):
 *   updateGeometry            :327-517   -> hrt_update_geometry
 *   buildAccelerationStructure:519-532   -> hrt_build_accel
 *   launchDirectRays          :813-870   -> hrt_launch_direct
 *   launchDiffuseRays         :872-1002  -> hrt_launch_diffuse (uploads radiation_out first)
 *   getRadiationResults       :1119-1143 -> hrt_get_results
 *   zero/copy/upload          :1168-1250 -> hrt_zero_* / hrt_copy_scatter_to_radiation / hrt_upload_radiation_out
 *   updateSkyModel            :744       -> hrt_update_sky_model
 *   launchCameraRays          :1004      -> hrt_launch_camera
 *   launchPixelLabelRays      :1071      -> hrt_launch_pixel_labels
 *   getCameraResults          :1145      -> hrt_get_camera_results
 *   zeroCameraPixelBuffers    :1207      -> hrt_zero_camera_pixel_buffers
 */
#include "GB300Backend.h"

#include <algorithm>
#include <iostream>
#include <string>

namespace helios {

GB300Backend::GB300Backend(int device) : device_(device) {}

GB300Backend::~GB300Backend() { shutdown(); }

void GB300Backend::check(int rc, const char *where) const {
    if (rc != HRT_OK) {
        helios_runtime_error(std::string("ERROR (GB300Backend::") + where + "): " +
                             (ctx_ ? hrt_last_error(ctx_) : "no device context") + " (code " + std::to_string(rc) + ")");
    }
}

void GB300Backend::initialize() {
    if (ctx_) return;
    check(hrt_create(&ctx_, device_), "initialize");
}

void GB300Backend::shutdown() {
    if (ctx_) {
        hrt_destroy(ctx_);
        ctx_ = nullptr;
    }
}

void GB300Backend::updateGeometry(const RayTracingGeometry &geometry) {
    validateGeometryBeforeUpload(geometry);
    std::vector<int8_t> twosided(geometry.twosided_flags.begin(), geometry.twosided_flags.end());
    std::vector<float> bbox;
    bbox.reserve(geometry.bboxes.vertices.size() * 3);
    for (const auto &v : geometry.bboxes.vertices) {
        bbox.push_back(v.x);
        bbox.push_back(v.y);
        bbox.push_back(v.z);
    }
    hrt_geometry g{};
    g.n = (int32_t)geometry.primitive_count;
    g.transform = geometry.transform_matrices.data();
    g.type = geometry.primitive_types.data();
    g.twosided = twosided.data();
    g.nbbox = (int32_t)geometry.bbox_count;
    g.bbox_vertices = bbox.empty() ? nullptr : bbox.data();
    g.periodic_x = geometry.periodic_flag.x;
    g.periodic_y = geometry.periodic_flag.y;
    if (!voxel_lad_.empty()) {
        if (voxel_lad_.size() != geometry.primitive_count)
            helios_runtime_error("ERROR (GB300Backend::updateGeometry): voxel leaf area density has " +
                                 std::to_string(voxel_lad_.size()) + " entries for " +
                                 std::to_string(geometry.primitive_count) + " primitives");
        g.voxel_lad = voxel_lad_.data();
    }
    // Texture masks: bool texels to bytes, the packed uv_data (4 entries per textured primitive
    // in primitive order, RadiationModel.cpp:6210-6222) to 4 corners per primitive.
    std::vector<uint8_t> mask_bytes(geometry.mask_data.begin(), geometry.mask_data.end());
    std::vector<int32_t> mask_size;
    for (const auto &sz : geometry.mask_sizes) {
        mask_size.push_back(sz.x);
        mask_size.push_back(sz.y);
    }
    std::vector<float> uv;
    if (!geometry.mask_sizes.empty() && geometry.mask_IDs.size() == geometry.primitive_count) {
        g.mask_id = geometry.mask_IDs.data();
        g.nmasks = (int32_t)geometry.mask_sizes.size();
        g.mask_size = mask_size.data();
        g.mask_data = mask_bytes.data();
        if (geometry.uv_IDs.size() == geometry.primitive_count) {
            uv.assign(geometry.primitive_count * 8, 0.f);
            size_t r = 0;
            for (size_t p = 0; p < geometry.primitive_count; ++p) {
                if (geometry.uv_IDs[p] < 0) continue;
                for (int v = 0; v < 4 && r < geometry.uv_data.size(); ++v, ++r) {
                    uv[p * 8 + 2 * v] = geometry.uv_data[r].x;
                    uv[p * 8 + 2 * v + 1] = geometry.uv_data[r].y;
                }
            }
            g.uv_id = geometry.uv_IDs.data();
            g.uv = uv.data();
        }
    }
    check(hrt_update_geometry(ctx_, &g), "updateGeometry");
    nprims_ = geometry.primitive_count;
}

void GB300Backend::buildAccelerationStructure() { check(hrt_build_accel(ctx_), "buildAccelerationStructure"); }

void GB300Backend::updateMaterials(const RayTracingMaterial &m) {
    check(hrt_update_materials(ctx_, (int32_t)m.num_sources, (int32_t)m.num_primitives, (int32_t)m.num_bands,
                               m.reflectivity.data(), m.transmissivity.data()),
          "updateMaterials");
    // translucent covers: is_glass / glass_n / glass_KL share the materials' layout
    const size_t count = m.num_sources * m.num_primitives * m.num_bands;
    const bool glass = m.is_glass.size() == count && m.glass_n.size() == count && m.glass_KL.size() == count &&
                       std::any_of(m.is_glass.begin(), m.is_glass.end(), [](char g) { return g != 0; });
    std::vector<int8_t> is_glass;
    if (glass) is_glass.assign(m.is_glass.begin(), m.is_glass.end());
    check(hrt_update_glass(ctx_, glass ? (int32_t)m.num_sources : 0, (int32_t)m.num_primitives,
                           glass ? (int32_t)m.num_bands : 0, glass ? is_glass.data() : nullptr,
                           glass ? m.glass_n.data() : nullptr, glass ? m.glass_KL.data() : nullptr),
          "updateMaterials");
}

void GB300Backend::updateSources(const std::vector<RayTracingSource> &sources) {
    std::vector<hrt_source> s(sources.size());
    for (size_t i = 0; i < sources.size(); ++i) {
        s[i].type = sources[i].type;
        s[i].position[0] = sources[i].position.x;
        s[i].position[1] = sources[i].position.y;
        s[i].position[2] = sources[i].position.z;
        s[i].width[0] = sources[i].width.x;
        s[i].width[1] = sources[i].width.y;
        s[i].rotation[0] = sources[i].rotation.x;
        s[i].rotation[1] = sources[i].rotation.y;
        s[i].rotation[2] = sources[i].rotation.z;
    }
    check(hrt_update_sources(ctx_, (int32_t)s.size(), s.data()), "updateSources");
}

// Diffuse parameters travel with each launch (as in OptiX8Backend::launchDiffuseRays).
void GB300Backend::updateDiffuseRadiation(const std::vector<float> &, const std::vector<float> &,
                                          const std::vector<helios::vec3> &, const std::vector<float> &,
                                          const std::vector<float> &) {}

// What cameras see where their rays leave the scene.
void GB300Backend::updateSkyModel(const std::vector<helios::vec4> &sky_radiance_params,
                                  const std::vector<float> &camera_sky_radiance, const helios::vec3 &sun_direction,
                                  const std::vector<float> &solar_disk_radiance, float solar_disk_cos_angle,
                                  const std::vector<float> &camera_diffuse_flux,
                                  const std::vector<uint32_t> &band_emission_flag) {
    const size_t B = std::max(sky_radiance_params.size(), camera_sky_radiance.size());
    std::vector<float> prague;
    for (const auto &v : sky_radiance_params) {
        prague.push_back(v.x);
        prague.push_back(v.y);
        prague.push_back(v.z);
        prague.push_back(v.w);
    }
    auto arr = [B](const std::vector<float> &v) { return v.size() >= B && B > 0 ? v.data() : nullptr; };
    hrt_sky_model m{};
    m.sky_radiance_params = prague.size() >= 4 * B && B > 0 ? prague.data() : nullptr;
    m.camera_sky_radiance = arr(camera_sky_radiance);
    m.sun_direction[0] = sun_direction.x;
    m.sun_direction[1] = sun_direction.y;
    m.sun_direction[2] = sun_direction.z;
    m.solar_disk_radiance = arr(solar_disk_radiance);
    m.solar_disk_cos_angle = solar_disk_cos_angle;
    m.camera_diffuse_flux = arr(camera_diffuse_flux);
    m.band_emission_flag = band_emission_flag.size() >= B && B > 0 ? band_emission_flag.data() : nullptr;
    check(hrt_update_sky_model(ctx_, (int32_t)B, B ? &m : nullptr), "updateSkyModel");
}

hrt_camera GB300Backend::makeCamera(const RayTracingLaunchParams &p) const {
    hrt_camera c{};
    c.position[0] = p.camera_position.x;
    c.position[1] = p.camera_position.y;
    c.position[2] = p.camera_position.z;
    c.direction[0] = p.camera_direction.x;
    c.direction[1] = p.camera_direction.y;
    c.focal_length = p.camera_focal_length;
    c.lens_diameter = p.camera_lens_diameter;
    c.fov_aspect = p.camera_fov_aspect;
    c.viewplane_length = p.camera_viewplane_length;
    c.resolution[0] = p.camera_resolution_full.x;
    c.resolution[1] = p.camera_resolution_full.y;
    c.tile_offset[0] = p.camera_pixel_offset.x;
    c.tile_offset[1] = p.camera_pixel_offset.y;
    c.tile_resolution[0] = p.camera_resolution.x;
    c.tile_resolution[1] = p.camera_resolution.y;
    c.antialiasing = (int32_t)p.antialiasing_samples;
    c.seed = p.random_seed;
    c.camera_id = p.camera_id;
    return c;
}

hrt_launch GB300Backend::makeLaunch(const RayTracingLaunchParams &p, std::vector<uint8_t> &flags,
                                    std::vector<float> &peak, std::vector<float> &sky) const {
    flags.assign(p.band_launch_flag.begin(), p.band_launch_flag.end());
    for (const auto &d : p.diffuse_peak_dir) {
        peak.push_back(d.x);
        peak.push_back(d.y);
        peak.push_back(d.z);
    }
    for (const auto &v : p.sky_radiance_params) {
        sky.push_back(v.x);
        sky.push_back(v.y);
        sky.push_back(v.z);
        sky.push_back(v.w);
    }
    hrt_launch L{};
    L.launch_offset = p.launch_offset;
    L.launch_count = p.launch_count;
    L.rays_per_primitive = p.rays_per_primitive;
    L.random_seed = p.random_seed;
    L.nbands_global = p.num_bands_global;
    L.nbands_launch = p.num_bands_launch;
    L.band_launch_flag = flags.data();
    L.launch_face = p.launch_face;
    L.diffuse_flux = p.diffuse_flux.empty() ? nullptr : p.diffuse_flux.data();
    L.diffuse_extinction = p.diffuse_extinction.empty() ? nullptr : p.diffuse_extinction.data();
    L.diffuse_peak_dir = peak.empty() ? nullptr : peak.data();
    L.diffuse_dist_norm = p.diffuse_dist_norm.empty() ? nullptr : p.diffuse_dist_norm.data();
    L.sky_radiance_params = sky.empty() ? nullptr : sky.data();
    L.radiation_out_top = p.radiation_out_top.empty() ? nullptr : p.radiation_out_top.data();
    L.radiation_out_bottom = p.radiation_out_bottom.empty() ? nullptr : p.radiation_out_bottom.data();
    return L;
}

void GB300Backend::launchDirectRays(const RayTracingLaunchParams &p) {
    std::vector<uint8_t> flags;
    std::vector<float> peak, sky;
    hrt_launch L = makeLaunch(p, flags, peak, sky);
    L.pass_id = 0;
    check(hrt_launch_direct(ctx_, &L), "launchDirectRays");
}

void GB300Backend::launchDiffuseRays(const RayTracingLaunchParams &p) {
    std::vector<uint8_t> flags;
    std::vector<float> peak, sky;
    hrt_launch L = makeLaunch(p, flags, peak, sky);
    L.pass_id = 1 + p.scattering_iteration;
    check(hrt_launch_diffuse(ctx_, &L), "launchDiffuseRays");
}

void GB300Backend::launchCameraRays(const RayTracingLaunchParams &p) {
    hrt_camera c = makeCamera(p);
    check(hrt_launch_camera(ctx_, &c), "launchCameraRays");
    camera_image_ = p.camera_resolution_full;
}

void GB300Backend::launchPixelLabelRays(const RayTracingLaunchParams &p) {
    hrt_camera c = makeCamera(p);
    check(hrt_launch_pixel_labels(ctx_, &c), "launchPixelLabelRays");
    label_image_ = p.camera_resolution_full;
}

void GB300Backend::getRadiationResults(RayTracingResults &r) {
    const size_t m = nprims_ * launch_bands_;
    r.num_primitives = nprims_;
    r.num_bands = launch_bands_;
    r.radiation_in.assign(m, 0.f);
    r.radiation_out_top.assign(m, 0.f);
    r.radiation_out_bottom.assign(m, 0.f);
    r.scatter_buff_top.assign(m, 0.f);
    r.scatter_buff_bottom.assign(m, 0.f);
    if (m == 0) return;
    check(hrt_get_results(ctx_, r.radiation_in.data(), r.radiation_out_top.data(), r.radiation_out_bottom.data(),
                          r.scatter_buff_top.data(), r.scatter_buff_bottom.data()),
          "getRadiationResults");
    // Camera-weighted scatter: the camera materials are the band materials here, so a pass's
    // camera scatter is its scatter (RadiationModel reads both right after the same launches).
    r.scatter_buff_top_cam = r.scatter_buff_top;
    r.scatter_buff_bottom_cam = r.scatter_buff_bottom;
}

void GB300Backend::getCameraResults(std::vector<float> &pixel_data, std::vector<uint> &pixel_labels,
                                    std::vector<float> &pixel_depths, uint, const helios::int2 &resolution) {
    const size_t npx = (size_t)std::max(resolution.x, 0) * (size_t)std::max(resolution.y, 0);
    if (npx == 0) return;
    if (camera_image_.x == resolution.x && camera_image_.y == resolution.y) {
        pixel_data.assign(npx * launch_bands_, 0.f);
        check(hrt_get_camera_results(ctx_, pixel_data.data(), nullptr, nullptr, resolution.x, resolution.y),
              "getCameraResults");
    }
    if (label_image_.x == resolution.x && label_image_.y == resolution.y) {
        std::vector<uint32_t> labels(npx, 0u);
        pixel_depths.assign(npx, 0.f);
        check(hrt_get_camera_results(ctx_, nullptr, labels.data(), pixel_depths.data(), resolution.x, resolution.y),
              "getCameraResults");
        pixel_labels.assign(labels.begin(), labels.end());
    }
}

void GB300Backend::zeroRadiationBuffers(size_t launch_band_count) {
    check(hrt_zero_radiation_buffers(ctx_, launch_band_count), "zeroRadiationBuffers");
    launch_bands_ = launch_band_count;
}

void GB300Backend::zeroScatterBuffers() { check(hrt_zero_scatter_buffers(ctx_), "zeroScatterBuffers"); }

void GB300Backend::zeroCameraPixelBuffers(const helios::int2 &resolution) {
    check(hrt_zero_camera_pixel_buffers(ctx_, resolution.x, resolution.y), "zeroCameraPixelBuffers");
    label_image_ = resolution;
}

void GB300Backend::copyScatterToRadiation() { check(hrt_copy_scatter_to_radiation(ctx_), "copyScatterToRadiation"); }

void GB300Backend::uploadRadiationOut(const std::vector<float> &top, const std::vector<float> &bottom) {
    size_t n = std::max(top.size(), bottom.size());
    check(hrt_upload_radiation_out(ctx_, top.empty() ? nullptr : top.data(), bottom.empty() ? nullptr : bottom.data(), n),
          "uploadRadiationOut");
}

void GB300Backend::zeroCameraScatterBuffers(size_t) {}

void GB300Backend::uploadSourceFluxes(const std::vector<float> &fluxes) {
    check(hrt_upload_source_fluxes(ctx_, fluxes.data(), fluxes.size()), "uploadSourceFluxes");
}

void GB300Backend::uploadSourceFluxesCam(const std::vector<float> &) {}

void GB300Backend::queryGPUMemory() const {
    size_t f = 0, t = 0;
    check(hrt_query_memory(ctx_, &f, &t), "queryGPUMemory");
    std::cout << "GPU memory: " << f / (1024.0 * 1024.0) << " MB free / " << t / (1024.0 * 1024.0) << " MB total"
              << std::endl;
}

std::string GB300Backend::getBackendName() const { return hrt_backend_name(); }

}  // namespace helios
