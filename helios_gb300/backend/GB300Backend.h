/** GB300Backend.h -- helios::RayTracingBackend implemented on libhrt (include/hrt.h).
 *
 * Drop-in for the radiation plugin: RadiationModel, the Context and downstream
 * plug-ins stay unchanged.  The class is compiled inside the Helios tree against
 * plugins/radiation/include/RayTracingBackend.h and injected with
 *     auto be = std::make_unique<helios::GB300Backend>();
 *     be->initialize();
 *     auto radiation = helios::RadiationModel::createWithBackend(&context, std::move(be));
 * (RadiationModel.h:730).  Every virtual forwards to one hrt_* call; a non-zero
 * return code becomes helios_runtime_error with the library's message.
 * Cameras render with the band materials (no per-camera spectral weighting) and without
 * specular highlights.
 */
#ifndef HELIOS_GB300_BACKEND_H
#define HELIOS_GB300_BACKEND_H

#include "RayTracingBackend.h"
#include "hrt.h"

namespace helios {

class GB300Backend : public RayTracingBackend {
public:
    explicit GB300Backend(int device = 0);
    ~GB300Backend() override;

    void initialize() override;
    void shutdown() override;
    void updateGeometry(const RayTracingGeometry &geometry) override;
    void buildAccelerationStructure() override;
    void updateMaterials(const RayTracingMaterial &materials) override;
    void updateSources(const std::vector<RayTracingSource> &sources) override;
    void updateDiffuseRadiation(const std::vector<float> &flux, const std::vector<float> &extinction,
                                const std::vector<helios::vec3> &peak_dir, const std::vector<float> &dist_norm,
                                const std::vector<float> &sky_energy) override;
    void updateSkyModel(const std::vector<helios::vec4> &sky_radiance_params, const std::vector<float> &camera_sky_radiance,
                        const helios::vec3 &sun_direction, const std::vector<float> &solar_disk_radiance,
                        float solar_disk_cos_angle, const std::vector<float> &camera_diffuse_flux,
                        const std::vector<uint32_t> &band_emission_flag) override;
    void launchDirectRays(const RayTracingLaunchParams &params) override;
    void launchDiffuseRays(const RayTracingLaunchParams &params) override;
    void launchCameraRays(const RayTracingLaunchParams &params) override;
    void launchPixelLabelRays(const RayTracingLaunchParams &params) override;
    void getRadiationResults(RayTracingResults &results) override;
    void getCameraResults(std::vector<float> &pixel_data, std::vector<uint> &pixel_labels,
                          std::vector<float> &pixel_depths, uint camera_id, const helios::int2 &resolution) override;
    void zeroRadiationBuffers(size_t launch_band_count) override;
    void zeroScatterBuffers() override;
    void zeroCameraPixelBuffers(const helios::int2 &resolution) override;
    void copyScatterToRadiation() override;
    void uploadRadiationOut(const std::vector<float> &radiation_out_top,
                            const std::vector<float> &radiation_out_bottom) override;
    void zeroCameraScatterBuffers(size_t launch_band_count) override;
    void uploadSourceFluxes(const std::vector<float> &fluxes) override;
    void uploadSourceFluxesCam(const std::vector<float> &fluxes_cam) override;
    void queryGPUMemory() const override;
    std::string getBackendName() const override;

    //! Leaf area density (m^2/m^3) of each primitive, read for voxels (type 4) at the next
    //! updateGeometry.  RayTracingGeometry carries none; a model with voxels sets it first.
    void setVoxelLeafAreaDensity(const std::vector<float> &lad) { voxel_lad_ = lad; }

private:
    void check(int rc, const char *where) const;
    hrt_launch makeLaunch(const RayTracingLaunchParams &p, std::vector<uint8_t> &flags, std::vector<float> &peak,
                          std::vector<float> &sky) const;
    hrt_camera makeCamera(const RayTracingLaunchParams &p) const;

    int device_;
    hrt_context *ctx_ = nullptr;
    size_t nprims_ = 0;
    size_t launch_bands_ = 0;
    std::vector<float> voxel_lad_;
    helios::int2 camera_image_{0, 0};  // resolution of the camera image on the device
    helios::int2 label_image_{0, 0};   // resolution of the pixel labels on the device
};

}  // namespace helios

#endif
