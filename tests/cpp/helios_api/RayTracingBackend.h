/* RayTracingBackend.h -- test stand-in for the reference's ray-tracing backend interface.
 *
 * The C++ drop-in adapter (helios_gb300/backend/GB300Backend.{h,cpp}) is written against
 * the reference's plugins/radiation/include/RayTracingBackend.h (class
 * helios::RayTracingBackend, :42-317) and RayTracingTypes.h (the RayTracingGeometry /
 * Material / Source / LaunchParams / Results structs, :40-271).  Those headers are not on a
 * GPU machine, so the adapter's GPU test compiles it against this file instead: the members the
 * adapter reads or writes, with the reference's names and element types (the interface has
 * to be alike for the same adapter source to compile against both), and nothing else.  On a
 * machine with the reference tree, tests/test_backend_adapter.py also compiles the adapter
 * against the reference's own headers.
 */
#ifndef HRT_TEST_RAYTRACINGBACKEND_H
#define HRT_TEST_RAYTRACINGBACKEND_H

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

typedef unsigned int uint;

namespace helios {

struct vec2 {
    float x = 0.f, y = 0.f;
};
struct vec3 {
    float x = 0.f, y = 0.f, z = 0.f;
};
struct vec4 {
    float x = 0.f, y = 0.f, z = 0.f, w = 0.f;
};
struct int2 {
    int x = 0, y = 0;
};

// Errors surface as std::runtime_error, as the reference's helper does (core/include/global.h:102).
inline void helios_runtime_error(const std::string &message) { throw std::runtime_error(message); }

struct PrimitiveTypeGeometry {
    std::vector<vec3> vertices;  // periodic wall quads: 4 corners each
    size_t count = 0;
};

struct RayTracingGeometry {
    std::vector<float> transform_matrices;  // [n*16] row-major
    std::vector<uint> primitive_types;      // 0 patch, 1 triangle, 2 disk, 3 tile, 4 voxel
    std::vector<char> twosided_flags;
    PrimitiveTypeGeometry bboxes;
    std::vector<bool> mask_data;
    std::vector<int2> mask_sizes;
    std::vector<int> mask_IDs;
    std::vector<vec2> uv_data;
    std::vector<int> uv_IDs;
    vec2 periodic_flag;
    size_t primitive_count = 0;
    size_t bbox_count = 0;
};

struct RayTracingMaterial {
    std::vector<float> reflectivity;    // [source][primitive][band]
    std::vector<float> transmissivity;
    std::vector<float> glass_n;
    std::vector<float> glass_KL;
    std::vector<char> is_glass;
    size_t num_bands = 0;
    size_t num_sources = 0;
    size_t num_primitives = 0;
};

struct RayTracingSource {
    vec3 position;
    vec3 rotation;
    vec2 width;
    uint type = 0;
};

struct RayTracingLaunchParams {
    uint launch_offset = 0;
    uint launch_count = 0;
    uint rays_per_primitive = 0;
    uint random_seed = 0;
    uint num_bands_global = 0;
    uint num_bands_launch = 0;
    std::vector<bool> band_launch_flag;
    uint scattering_iteration = 0;
    uint launch_face = 0;
    uint camera_id = 0;
    vec3 camera_position;
    vec2 camera_direction;
    float camera_focal_length = 0.f;
    float camera_lens_diameter = 0.f;
    float camera_fov_aspect = 0.f;
    int2 camera_resolution;
    uint antialiasing_samples = 1;
    int2 camera_pixel_offset;
    float camera_viewplane_length = 0.f;
    int2 camera_resolution_full;
    std::vector<float> diffuse_flux;
    std::vector<float> diffuse_extinction;
    std::vector<vec3> diffuse_peak_dir;
    std::vector<float> diffuse_dist_norm;
    std::vector<vec4> sky_radiance_params;
    std::vector<float> radiation_out_top;
    std::vector<float> radiation_out_bottom;
};

struct RayTracingResults {
    std::vector<float> radiation_in;
    std::vector<float> radiation_out_top;
    std::vector<float> radiation_out_bottom;
    std::vector<float> scatter_buff_top;
    std::vector<float> scatter_buff_bottom;
    std::vector<float> scatter_buff_top_cam;
    std::vector<float> scatter_buff_bottom_cam;
    size_t num_primitives = 0;
    size_t num_bands = 0;
};

class RayTracingBackend {
public:
    virtual ~RayTracingBackend() = default;
    virtual void initialize() = 0;
    virtual void shutdown() = 0;
    virtual void updateGeometry(const RayTracingGeometry &geometry) = 0;
    virtual void buildAccelerationStructure() = 0;
    virtual void updateMaterials(const RayTracingMaterial &materials) = 0;
    virtual void updateSources(const std::vector<RayTracingSource> &sources) = 0;
    virtual void updateDiffuseRadiation(const std::vector<float> &flux, const std::vector<float> &extinction,
                                        const std::vector<vec3> &peak_dir, const std::vector<float> &dist_norm,
                                        const std::vector<float> &sky_energy) = 0;
    virtual void updateSkyModel(const std::vector<vec4> &sky_radiance_params, const std::vector<float> &camera_sky_radiance,
                                const vec3 &sun_direction, const std::vector<float> &solar_disk_radiance,
                                float solar_disk_cos_angle, const std::vector<float> &camera_diffuse_flux,
                                const std::vector<uint32_t> &band_emission_flag) = 0;
    virtual void launchDirectRays(const RayTracingLaunchParams &params) = 0;
    virtual void launchDiffuseRays(const RayTracingLaunchParams &params) = 0;
    virtual void launchCameraRays(const RayTracingLaunchParams &params) = 0;
    virtual void launchPixelLabelRays(const RayTracingLaunchParams &params) = 0;
    virtual void getRadiationResults(RayTracingResults &results) = 0;
    virtual void getCameraResults(std::vector<float> &pixel_data, std::vector<uint> &pixel_labels,
                                  std::vector<float> &pixel_depths, uint camera_id, const int2 &resolution) = 0;
    virtual void zeroRadiationBuffers(size_t launch_band_count) = 0;
    virtual void zeroScatterBuffers() = 0;
    virtual void zeroCameraPixelBuffers(const int2 &resolution) = 0;
    virtual void copyScatterToRadiation() = 0;
    virtual void uploadRadiationOut(const std::vector<float> &radiation_out_top,
                                    const std::vector<float> &radiation_out_bottom) = 0;
    virtual void zeroCameraScatterBuffers(size_t launch_band_count) = 0;
    virtual void uploadSourceFluxes(const std::vector<float> &fluxes) = 0;
    virtual void uploadSourceFluxesCam(const std::vector<float> &fluxes_cam) = 0;
    virtual void queryGPUMemory() const = 0;
    virtual std::string getBackendName() const = 0;

protected:
    // Size checks before an upload (the reference runs its own in debug builds).
    void validateGeometryBeforeUpload(const RayTracingGeometry &g) const {
        const size_t n = g.primitive_count;
        if (g.transform_matrices.size() != 16 * n || g.primitive_types.size() != n || g.twosided_flags.size() != n)
            helios_runtime_error("RayTracingGeometry: per-primitive arrays do not match primitive_count");
        if (g.bboxes.vertices.size() != 4 * g.bbox_count)
            helios_runtime_error("RayTracingGeometry: periodic walls need 4 corners each");
    }
};

}  // namespace helios

#endif
