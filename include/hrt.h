/* hrt.h -- C ABI of libhrt, the GB300 (sm_103a) radiation-transfer engine.
 *
 * This is the drop-in boundary for the Helios radiation plugin.  The reference
 * talks to its ray tracers only through the abstract class
 * helios::RayTracingBackend (plugins/radiation/include/RayTracingBackend.h:42-317);
 * each entry point below replaces one of its virtuals, named in the comment
 * with the file:line of the declaration.  A C++ adapter that implements that
 * class on top of these functions lives in helios_gb300/backend/.
 *
 * Conventions
 *   - All pointers passed in are HOST pointers unless a name says otherwise;
 *     sizes are element counts.  The library copies inputs to device memory it
 *     owns; results are copied back into caller-provided host arrays.
 *   - Every function returns HRT_OK (0) or a negative HRT_E* code; the text of
 *     the last error of a context is returned by hrt_last_error().  The C++
 *     adapter turns a non-zero code into helios::helios_runtime_error, which is
 *     how the reference reports backend failures (core/include/global.h:102).
 *   - Radiation buffers are indexed [primitive * Nbands_launch + band_launch],
 *     materials [source * Nprims * Nbands_global + prim * Nbands_global + band]
 *     (plugins/radiation/include/BufferIndexing.h:216-252).
 *   - A context is used by one host thread at a time.  Calls are synchronous
 *     unless stated otherwise, as the reference backends are
 *     (OptiX8Backend.cpp:866,998).
 */
#ifndef HRT_H
#define HRT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HRT_OK 0
#define HRT_EINVAL -1      /* bad argument or call order */
#define HRT_ECUDA -2       /* CUDA runtime error */
#define HRT_ENOMEM -3      /* device allocation failed */
#define HRT_EDEVICE -4     /* device-side error word set (stack overflow, wrap limit) */
#define HRT_EUNSUPPORTED -5

typedef struct hrt_context hrt_context;

/* Geometry, the subset of helios::RayTracingGeometry (RayTracingTypes.h:40-155)
 * that the radiation solve reads.  Primitive types: 0 patch, 1 triangle, 2 disk,
 * 3 tile (traced as a patch), 4 voxel.  Periodic walls are the reference's
 * "bbox" primitives (type 5), passed separately as world-space quads.
 *
 * Disks are native unit disks scaled by their transform (the OptiX 6 semantics of
 * primitiveIntersection.cu:236-300; the reference's OptiX 8 backend has none).
 * Voxels are axis-aligned boxes filled with a turbid medium of leaves with a spherical
 * angle distribution: extinction G * LAD with G = 0.5, free-path interception drawn per
 * (ray, voxel), isotropic launch (pairs of opposite directions), leaves scattering
 * rho + tau isotropically.  Their fluxes are per unit LEAF area (LAD x volume).  The
 * reference has no voxel radiation physics (OptiX 6 rayHit.cu:278-290 is commented
 * out), so these are this library's definitions. */
typedef struct {
    int32_t n;                    /* primitive_count */
    const float *transform;       /* [n*16] row-major 4x4 (transform_matrices) */
    const uint32_t *type;         /* [n] primitive_types */
    const int8_t *twosided;       /* [n] twosided_flags: 0 one-sided, 1 two-sided, 2, 3 (skip); voxels are two-sided */
    int32_t nbbox;                /* bbox_count: 0, 2 or 4 periodic walls */
    const float *bbox_vertices;   /* [nbbox*4*3] wall corners (bboxes.vertices) */
    float periodic_x, periodic_y; /* periodic_flag */
    const float *voxel_lad;       /* [n] leaf area density (m^2/m^3) read for voxels; may be NULL without voxels */
    /* Texture masks (RayTracingGeometry mask_IDs / uv_IDs / uv_data / mask_sizes / mask_data,
     * RayTracingTypes.h:72-77): a masked patch or triangle is hit, and launches rays, only
     * where its mask texel is nonzero.  mask_id NULL or nmasks 0: no masks. */
    const int32_t *mask_id;       /* [n] mask of each primitive, -1 none */
    const int32_t *uv_id;         /* [n] >= 0: uv holds the primitive's texture coordinates, or NULL */
    const float *uv;              /* [n*8] (u,v) of the canonical corners 0..3 (triangles: 0..2), or NULL */
    int32_t nmasks;
    const int32_t *mask_size;     /* [nmasks*2] width, height */
    const uint8_t *mask_data;     /* masks one after another, each row-major [y][x] */
} hrt_geometry;

/* helios::RayTracingSource (RayTracingTypes.h:189-196) without the flux vectors,
 * which travel through hrt_upload_source_fluxes(). */
typedef struct {
    uint32_t type;        /* 0 collimated, 1 sphere, 2 sun sphere, 3 rectangle, 4 disk */
    float position[3];    /* direction toward the source (collimated) or centre */
    float width[2];       /* diameter / rectangle sides */
    float rotation[3];    /* Euler angles (rectangle and disk sources) */
} hrt_source;

/* helios::RayTracingLaunchParams (RayTracingTypes.h:201-250), radiation fields. */
typedef struct {
    uint32_t launch_offset;             /* first primitive */
    uint32_t launch_count;              /* number of primitives */
    uint32_t rays_per_primitive;        /* split into floor(sqrt(n)) x (n / floor(sqrt(n))) strata */
    uint32_t random_seed;               /* Philox key word 0 */
    uint32_t pass_id;                   /* Philox key word 1 (0 direct, 1 primary diffuse, 2+s scatter s) */
    uint32_t nbands_global;
    uint32_t nbands_launch;             /* buffer stride */
    const uint8_t *band_launch_flag;    /* [nbands_global] */
    uint32_t launch_face;               /* diffuse: 1 top, 0 bottom */
    const float *diffuse_flux;          /* [nbands_launch] */
    const float *diffuse_extinction;    /* [nbands_launch] power-law K, or NULL */
    const float *diffuse_peak_dir;      /* [nbands_launch*3] or NULL */
    const float *diffuse_dist_norm;     /* [nbands_launch] or NULL */
    const float *sky_radiance_params;   /* [nbands_launch*4] Prague parameters, or NULL */
    const float *radiation_out_top;     /* [n*nbands_launch] uploaded before a diffuse launch, or NULL */
    const float *radiation_out_bottom;  /* [n*nbands_launch] or NULL */
} hrt_launch;

/* One whole RadiationModel::runBand() (RadiationModel.cpp:3470-4663) executed on
 * the device: direct pass, emission source term, primary diffuse pass and the
 * scattering iterations, with every intermediate buffer kept in HBM. */
/* Camera of a launch (the camera fields of RayTracingLaunchParams, RayTracingTypes.h:220-234).
 * A camera ray of pixel (ii, jj) leaves a point of the lens toward the focal plane through
 * the pixel's sub-pixel sample (OptiX8DeviceCode.cu:1665-1738); pixel (0, 0) is the top left.
 * The outputs are read by hrt_run_band only (the granular calls use hrt_get_camera_results). */
typedef struct {
    float position[3];            /* camera_position */
    float direction[2];           /* camera_direction: zenith and azimuth (radians) of lookat - position */
    float focal_length;           /* camera_focal_length: distance to the focal plane */
    float lens_diameter;          /* camera_lens_diameter; 0 = pinhole */
    float fov_aspect;             /* camera_fov_aspect = HFOV / VFOV */
    float viewplane_length;       /* camera_viewplane_length = 0.5 / tan(HFOV / 2) */
    int32_t resolution[2];        /* camera_resolution_full: width, height */
    int32_t tile_offset[2];       /* camera_pixel_offset: first pixel of this launch */
    int32_t tile_resolution[2];   /* camera_resolution: pixels of this launch; 0 = the whole image */
    int32_t antialiasing;         /* antialiasing_samples: rays per pixel */
    uint32_t seed;                /* random_seed */
    uint32_t camera_id;           /* camera_id */
    float *pixels;                /* out [height*width*Bl] radiance, pixel-major, or NULL */
    uint32_t *labels;             /* out [height*width] hit primitive + 1 (0 = sky), or NULL */
    float *depths;                /* out [height*width] depth along the view axis (-1 = sky), or NULL */
} hrt_camera;

/* What cameras see where their rays leave the scene (RayTracingBackend::updateSkyModel,
 * RayTracingBackend.h:129): per launched band.  Any array may be NULL (nothing seen). */
typedef struct {
    const float *sky_radiance_params;   /* [Bl*4] Prague parameters of the camera sky */
    const float *camera_sky_radiance;   /* [Bl] sky radiance on a miss that sees no source */
    float sun_direction[3];             /* unit vector toward the sun */
    const float *solar_disk_radiance;   /* [Bl] radiance of the solar disk (collimated / sun-sphere sources) */
    float solar_disk_cos_angle;         /* a miss within this cosine of the sun sees the disk */
    const float *camera_diffuse_flux;   /* [Bl] sky flux of emission bands, seen as isotropic radiance */
    const uint32_t *band_emission_flag; /* [Bl] */
} hrt_sky_model;

typedef struct {
    int32_t nbands_global;
    const uint8_t *band_launch;         /* [nbands_global] bands run by this call */
    int32_t nsources;
    const hrt_source *sources;          /* [nsources], or NULL to keep the sources already set */
    const float *source_flux;           /* [nsources*Bl], or NULL to keep the fluxes already set */
    const float *rho, *tau;             /* [nsources*n*nbands_global], or NULL to keep the materials already set */
    const float *diffuse_flux;          /* [Bl] */
    const float *diffuse_extinction;    /* [Bl] or NULL */
    const float *diffuse_peak_dir;      /* [Bl*3] or NULL */
    const float *diffuse_dist_norm;     /* [Bl] or NULL */
    const float *sky_radiance_params;   /* [Bl*4] or NULL */
    const int32_t *direct_rays;         /* [Bl] directRayCount per band */
    const int32_t *diffuse_rays;        /* [Bl] diffuseRayCount per band */
    const int32_t *scattering_depth;    /* [Bl] */
    const uint8_t *emission;            /* [Bl] emission flag per band */
    const float *emissivity;            /* [n*Bl], or NULL to reuse the array of an earlier call */
    const float *temperature;           /* [n] kelvin, or NULL to reuse the array of an earlier call */
    uint32_t seed;
    /* > 0: FP64 convergence check after every scattering iteration (no counterpart in the
     * reference, which always runs scattering_depth iterations).  A band stops once the
     * area-weighted power its last iteration scattered, not yet propagated, is at most
     * scatter_tolerance times its total (absorbed + that); that power stays in the flux
     * as at the depth limit.  0 runs the reference's fixed iteration count. */
    double scatter_tolerance;
    /* Cameras rendered after the solve (RadiationModel.cpp:4358-4616): each sees every
     * primitive's scattered and emitted radiation accumulated over all passes.  Rendered only
     * when scattering is enabled and something radiates, as in the reference; else the pixels
     * are zero.  camera_sky NULL: the cameras see nothing where their rays leave the scene. */
    int32_t ncameras;
    const hrt_camera *cameras;
    const hrt_sky_model *camera_sky;
} hrt_band_solve;

/* ---- lifecycle: RayTracingBackend::initialize / shutdown (RayTracingBackend.h:54,61) */
int hrt_create(hrt_context **out, int device);
int hrt_destroy(hrt_context *ctx);
const char *hrt_last_error(const hrt_context *ctx);
/* Run all work of this context on `stream` (a cudaStream_t), or NULL for the
 * context's own stream. */
int hrt_set_stream(hrt_context *ctx, void *stream);

/* ---- RayTracingBackend::updateGeometry (RayTracingBackend.h:73) */
int hrt_update_geometry(hrt_context *ctx, const hrt_geometry *g);
/* ---- RayTracingBackend::buildAccelerationStructure (RayTracingBackend.h:81) */
int hrt_build_accel(hrt_context *ctx);
/* ---- RayTracingBackend::updateMaterials (RayTracingBackend.h:90) */
int hrt_update_materials(hrt_context *ctx, int32_t nsources, int32_t nprims, int32_t nbands_global,
                         const float *rho, const float *tau);
/* ---- The glass part of RayTracingBackend::updateMaterials (RayTracingBackend.h:90): translucent
 * covers (RayTracingMaterial glass_n / glass_KL / is_glass, RayTracingTypes.h:173-178, as
 * OptiX8Backend::updateMaterials uploads them, OptiX8Backend.cpp:581-597).  Arrays are
 * [nsources][nprims][nbands_global] like the materials.  A primitive that is glass in EVERY band of
 * a launch is a cover for that launch's rays of the source: rays pass it, each cover crossed before
 * a ray's end attenuates the ray by the Fresnel + Bouguer transmittance of one sheet per band and
 * takes its absorbed and reflected shares of the flux reaching it; covers are taken in order of
 * distance (the reference visits them in any-hit order).  is_glass NULL or all zero: no covers.
 * At most 32 sources and 16 launched bands; the batched sweep refuses scenes with covers. */
int hrt_update_glass(hrt_context *ctx, int32_t nsources, int32_t nprims, int32_t nbands_global, const int8_t *is_glass,
                     const float *glass_n, const float *glass_kl);
/* ---- RayTracingBackend::updateSources (RayTracingBackend.h:99) */
int hrt_update_sources(hrt_context *ctx, int32_t nsources, const hrt_source *sources);
/* ---- RayTracingBackend::uploadSourceFluxes (RayTracingBackend.h:247) [source*Bl + band] */
int hrt_upload_source_fluxes(hrt_context *ctx, const float *fluxes, size_t count);
/* ---- RayTracingBackend::launchDirectRays (RayTracingBackend.h:139) */
int hrt_launch_direct(hrt_context *ctx, const hrt_launch *p);
/* ---- RayTracingBackend::launchDiffuseRays (RayTracingBackend.h:146) */
int hrt_launch_diffuse(hrt_context *ctx, const hrt_launch *p);
/* ---- Surface energy balance: the step after the radiation solve (EnergyBalanceModel::run,
 * plugins/energybalance/src/EnergyBalanceModel.cu:34-125 and :466-505).  Per primitive, the
 * temperature T that closes R = Nsides eps sigma T^4 + QH + QL + Qother + storage, by the
 * reference's secant iteration (from the previous temperature and 400 K, relative step 1e-4,
 * at most 100 steps).  All arrays [n]. */
typedef struct {
    const float *air_temperature;      /* Ta (K) */
    const float *air_vapor_pressure;   /* ea (Pa) */
    const float *air_pressure;         /* Pa */
    const float *bl_conductance;       /* gH: boundary-layer conductance to heat (mol/m^2/s) */
    const float *moisture_conductance; /* gS: surface / stomatal conductance to vapour (mol/m^2/s) */
    const float *emissivity;           /* thermal emissivity */
    const float *other_flux;           /* Qother (W/m^2) */
    const float *heat_capacity;        /* J/m^2/K, used when dt > 0 */
    const float *surface_humidity;     /* relative humidity at the evaporating surface */
    const float *stomatal_sidedness;   /* fraction of the stomata on the second face */
    const uint8_t *nsides;             /* emitting faces: 1 or 2 */
    float dt;                          /* s; > 0 adds the heat-storage term */
    float temperature_default;         /* K, kept where the solution is not finite */
} hrt_surface;

/* net_radiation NULL: the sum over bands of the last hrt_run_band's fluxes (device-resident).
 * temperature NULL: the context's resident emission temperature.  The solved temperature
 * becomes the resident emission temperature, which the next hrt_run_band with temperature =
 * NULL emits with.  temperature_out [n] and fluxes_out [n*5] (sensible, latent, storage, net
 * radiation, vapour pressure deficit / P) may be NULL.  hrt_last_stats [3]: primitives whose
 * iteration did not converge. */
int hrt_energy_balance(hrt_context *ctx, int32_t n, const hrt_surface *s, const float *net_radiation,
                       const float *temperature, float *temperature_out, float *fluxes_out);

/* Radiation and energy balance coupled on the device: repeat { hrt_run_band(s) with the
 * resident temperatures; hrt_energy_balance on its fluxes } until no temperature changes by
 * more than tolerance_K or max_iterations solves have run.  The first solve uses s as given
 * (its temperature, if any); later ones keep materials, sources and emissivities resident.
 * flux_out [n*Bl] is the last solve's flux, temperature_out [n] the final temperatures. */
int hrt_run_coupled(hrt_context *ctx, const hrt_band_solve *s, const hrt_surface *surface, int32_t max_iterations,
                    float tolerance_K, float *flux_out, float *temperature_out, int32_t *iterations_out);

/* ---- Scene ingestion: the geometry of Context::loadPLY / loadOBJ / loadXML
 * (core/src/Context_fileIO.cpp:3633-3908, 3995-4340, 1260-2230) as primitive arrays for
 * hrt_update_geometry or hrt_server_add_scene.  PLY (ascii and binary little-endian) and OBJ
 * give triangles: up-axis remap, base moved to z = 0 (PLY), scaled to `height` (> 0), rotated
 * by (elevation, azimuth) as rotatePoint does, moved to `origin`, polygons fan-triangulated and
 * degenerate triangles dropped; OBJ triangles are grouped by material name, with the material's
 * Kd colour.  XML gives patches, triangles, voxels and disks with their <transform> (triangles
 * also from <vertices>) and scalar primitive data (<data_float>, <data_double>, <data_int>,
 * <data_uint>).  Texture images, compound objects and materials beyond Kd are not read. */
typedef struct hrt_scene_file hrt_scene_file;
typedef struct {
    float origin[3];
    float height;                 /* > 0: scale the model to this height (PLY, OBJ) */
    float rotation[2];            /* elevation, azimuth (radians) */
    int32_t up_axis;              /* 0 XUP, 1 YUP, 2 ZUP */
    float default_color[3];       /* colour of triangles without one */
} hrt_load_options;
/* opt NULL: origin 0, no scaling or rotation, ZUP, blue.  On failure *out is NULL and
 * hrt_scene_last_error() (per thread) says why. */
int hrt_scene_load(const char *path, const hrt_load_options *opt, hrt_scene_file **out);
const char *hrt_scene_last_error(void);
int64_t hrt_scene_count(const hrt_scene_file *f);
/* transform [n*16], type [n], twosided [n], color [n*3]; any may be NULL */
int hrt_scene_arrays(const hrt_scene_file *f, float *transform, uint32_t *type, int8_t *twosided, float *color);
/* primitive data labels, one per line; returns the buffer size needed */
size_t hrt_scene_data_labels(const hrt_scene_file *f, char *buf, size_t len);
/* values [n] of a primitive data label (NaN where a primitive has none) */
int hrt_scene_data(const hrt_scene_file *f, const char *label, double *values);
void hrt_scene_free(hrt_scene_file *f);

/* ---- RayTracingBackend::updateSkyModel (RayTracingBackend.h:129) */
int hrt_update_sky_model(hrt_context *ctx, int32_t nbands, const hrt_sky_model *m);
/* ---- RayTracingBackend::launchCameraRays (RayTracingBackend.h:153): adds the radiance of every
 * pixel of the launch's tile, as seen through radiation_out and the sources, to the camera buffer.
 * The buffer is zeroed when the camera id or band count differs from the previous launch, or after
 * hrt_zero_radiation_buffers (the OptiX8Backend rule, OptiX8Backend.cpp:1023-1037). */
int hrt_launch_camera(hrt_context *ctx, const hrt_camera *cam);
/* ---- RayTracingBackend::launchPixelLabelRays (RayTracingBackend.h:160): one ray through each
 * pixel centre of the tile; label = hit primitive + 1, depth along the view axis, -1 on a miss. */
int hrt_launch_pixel_labels(hrt_context *ctx, const hrt_camera *cam);
/* ---- RayTracingBackend::zeroCameraPixelBuffers (RayTracingBackend.h:210) */
int hrt_zero_camera_pixel_buffers(hrt_context *ctx, int32_t width, int32_t height);
/* ---- RayTracingBackend::getCameraResults (RayTracingBackend.h:182): pixels [height*width*Bl]
 * (pixel-major), labels and depths [height*width]; any pointer may be NULL. */
int hrt_get_camera_results(hrt_context *ctx, float *pixels, uint32_t *labels, float *depths, int32_t width,
                           int32_t height);
/* ---- RayTracingBackend::getRadiationResults (RayTracingBackend.h:171): any pointer may be NULL */
int hrt_get_results(hrt_context *ctx, float *radiation_in, float *radiation_out_top, float *radiation_out_bottom,
                    float *scatter_top, float *scatter_bottom);
/* ---- RayTracingBackend::zeroRadiationBuffers (RayTracingBackend.h:194) */
int hrt_zero_radiation_buffers(hrt_context *ctx, size_t launch_band_count);
/* ---- RayTracingBackend::zeroScatterBuffers (RayTracingBackend.h:199) */
int hrt_zero_scatter_buffers(hrt_context *ctx);
/* ---- RayTracingBackend::copyScatterToRadiation (RayTracingBackend.h:218) */
int hrt_copy_scatter_to_radiation(hrt_context *ctx);
/* ---- RayTracingBackend::uploadRadiationOut (RayTracingBackend.h:228) */
int hrt_upload_radiation_out(hrt_context *ctx, const float *top, const float *bottom, size_t count);
/* ---- RayTracingBackend::queryGPUMemory (RayTracingBackend.h:263) */
int hrt_query_memory(hrt_context *ctx, size_t *free_bytes, size_t *total_bytes);
/* ---- RayTracingBackend::getBackendName (RayTracingBackend.h:270) */
const char *hrt_backend_name(void);

/* ---- whole runBand on the device (RadiationModel::runBand, RadiationModel.cpp:3470-4663).
 * flux_out: host [n*Bl] = radiation_in + scatter_top + scatter_bottom
 * (RadiationModel.cpp:4652), or NULL to leave the result on the device. */
int hrt_run_band(hrt_context *ctx, const hrt_band_solve *s, float *flux_out);
/* ---- many solves of one scene in one launch graph (no counterpart in the reference;
 * it replaces nsun*nbands separate runBand calls).  Channel c = sun*nbands + band is the
 * solve RadiationModel::runBand(band) would give with one collimated source toward
 * sun_dir[sun], source flux direct_flux[c], isotropic sky flux diffuse_flux[c], the same
 * ray counts, depth and seed; no emission.  Direct rays are traced per sun; every diffuse
 * and scattering pass is traced ONCE for all channels (the rays do not depend on the sun)
 * and each ray's hit is gathered for every channel.  The whole sweep is captured into a
 * CUDA graph on the first call of a given shape and replayed afterwards. */
typedef struct {
    int32_t nsun;
    const float *sun_dir;        /* [nsun*3] direction toward each sun */
    int32_t nbands;
    const float *direct_flux;    /* [nsun*nbands] (0 with the sun below the horizon) */
    const float *diffuse_flux;   /* [nsun*nbands] isotropic sky flux */
    const float *rho, *tau;      /* [n*nbands] */
    int32_t direct_rays, diffuse_rays, scattering_depth;
    uint32_t seed;
} hrt_sweep;
/* flux_out: host [n*nsun*nbands] (channel fastest), or NULL. */
int hrt_run_sweep(hrt_context *ctx, const hrt_sweep *s, float *flux_out);
/* ---- sweeps of several scenes in one launch graph (no counterpart in the reference).
 * ctxs[k] holds scene k (its geometry and BVH, built as for any solve; all on one device,
 * 4-wide trees); sweeps[k] is its sweep, as for hrt_run_sweep.  The recording launches run
 * one resident wave (no per-thread ray budget applies).  The graph, on
 * ctxs[0]'s stream, runs every scene's direct pass and channel bookkeeping, and traces each
 * diffuse or scattering pass of ALL scenes in ONE persistent recording launch whose ray ids
 * run over the scenes one after another (at most 32 scene chunks per pass).  Each scene's
 * channels equal its hrt_run_sweep (the same Philox rays; sums in the same fixed order).
 * flux_out[k]: host [n_k*nsun_k*nbands_k] or NULL (flux_out itself may be NULL).  Captured
 * on the first call of a shape and replayed; the call returns after the graph finished;
 * a device error of scene k is reported with its index. */
int hrt_run_sweep_multi(hrt_context *const *ctxs, const hrt_sweep *sweeps, int32_t nscenes, float *const *flux_out);

/* ---- continuous-batching server (no counterpart in the reference; a serving front end
 * for many radiation solves of uneven size).  Scenes are registered once (geometry and
 * one-source rho/tau for nbands_global bands).  Requests carry an arrival time (seconds
 * after hrt_server_start) and one runBand's parameters; a dispatcher thread admits them
 * in arrival order when the scene's device context is idle and its footprint fits in
 * hbm_budget_bytes (least-recently-used idle scenes are evicted; resident scenes keep
 * their BVH and buffers).  Arrived requests of the same scene with the same band set,
 * ray counts, depth and seed are batched (up to 64 requests, 256 channels) into one
 * hrt_run_sweep: direct rays per request sun, diffuse and scattering passes traced once.
 * Worker threads run the batches on per-scene CUDA streams, so solves of different
 * scenes overlap on the GPU.  A result depends only on the request, not on what else is
 * in flight (up to the order of FP64 sums). */
typedef struct hrt_server hrt_server;
typedef struct {
    uint64_t request_id;
    uint32_t scene_id;
    double arrival_s;
    const uint8_t *band_launch;   /* [nbands_global of the scene] */
    float sun_dir[3];             /* collimated source direction */
    const float *source_flux;     /* [Bl] */
    const float *diffuse_flux;    /* [Bl] isotropic sky */
    int32_t direct_rays, diffuse_rays, scattering_depth;
    uint32_t seed;
    int32_t keep_result;          /* keep the [n*Bl] flux for hrt_server_result */
} hrt_serve_request;
int hrt_server_create(hrt_server **out, int device, int workers, size_t hbm_budget_bytes);
int hrt_server_add_scene(hrt_server *s, uint32_t scene_id, const hrt_geometry *g, int32_t nbands_global,
                         const float *rho, const float *tau);
int hrt_server_submit(hrt_server *s, const hrt_serve_request *req);
int hrt_server_start(hrt_server *s);
int hrt_server_wait(hrt_server *s);
/* timing: [arrival, admit, done] seconds; checksum = sum of the request's flux values. */
int hrt_server_result(hrt_server *s, uint64_t request_id, float *flux_out, size_t count, double *timing,
                      double *checksum, uint64_t *rays);
/* out: [0] BVH builds, [1] evictions, [2] bytes accounted resident, [3] budget,
 * [4] batches run, [5] requests in them, [6] multi-scene groups run, [7] batches in them. */
int hrt_server_stats(hrt_server *s, double *out, int count);
int hrt_server_destroy(hrt_server *s);

/* Kernel-variant tuner (no counterpart in the reference).  The diffuse trace has
 * interchangeable variants (persistent threads with 4 or 3 resident blocks per SM, one
 * ray per thread); the first pass of each shape (rays per face, faces, bands, scene
 * size) of at least 2e7 rays times them on a sample of its rays and keeps the fastest
 * for later passes, solves and sweep graphs of that shape.  mode 1 (default) tunes,
 * 0 uses the fixed default, 2 forgets earlier choices and tunes again, 16 + v forces
 * variant v (1 binary nodes / 4 blocks per SM, 2 binary / 3, 3 one ray per thread,
 * 4 compressed 4-wide / 4, 5 compressed 4-wide / 3).  Variants give the same results up
 * to the order of FP64 sums. */
int hrt_set_tuning(hrt_context *ctx, int mode);
/* Share the GPU with other streams (no counterpart in the reference).  By default the
 * persistent diffuse trace runs one resident wave of blocks until every ray is done, so
 * kernels of other streams wait for it.  With rays_per_thread > 0 a thread takes at most
 * that many rays before its block retires; the launch has enough blocks for all rays and
 * the hardware interleaves them with other streams' blocks (by stream priority).
 * Results do not change.  0 restores the default. */
int hrt_set_ray_budget(hrt_context *ctx, uint32_t rays_per_thread);
/* Launch planning (the reference likewise splits a pass into launches of at most 65,535
 * primitives, the OptiX depth limit: OptiX8Backend.cpp:854-868, 985-1000).  Ray ids inside one trace launch
 * are 32-bit, so a pass whose primitives x rays per primitive x faces reaches 2^31 runs as
 * consecutive launches over primitive chunks; results do not depend on the chunking
 * beyond the order of FP64 sums.  hrt_plan_launch_chunks returns the number of launches
 * for `count` primitives of `rays_per_primitive` rays each (all faces) under `max_rays`
 * rays per launch (0: the library's 2^31), and the primitives per launch in
 * *prims_per_chunk; HRT_EUNSUPPORTED when one primitive's rays exceed a launch.  It is
 * pure host arithmetic.  hrt_set_launch_ray_limit lowers a context's limit (tests force
 * small scenes through several chunks with it); values above 2^31 are clamped. */
int64_t hrt_plan_launch_chunks(uint32_t count, uint64_t rays_per_primitive, uint64_t max_rays,
                               uint32_t *prims_per_chunk);
int hrt_set_launch_ray_limit(hrt_context *ctx, uint64_t max_rays);
/* Node visits one ray segment may make before traversal ends it and sets the bounds
 * bit of the device error word (a ray visits each node at most once, so the default,
 * 0, means 2n+64 and never fires on a valid tree).  Tests set a tiny budget to drive
 * the device error path: the next solve returns HRT_EDEVICE and clears the word. */
int hrt_set_visit_budget(hrt_context *ctx, uint32_t visits);
/* Text log of the tuner's trials and choices, one line per shape; returns the bytes
 * needed (including the terminating zero); buf may be NULL. */
size_t hrt_tuning_report(const hrt_context *ctx, char *buf, size_t len);
/* Statistics of the last hrt_run_band: [0] rays traced, [1] kernels launched,
 * [2] scattering iterations run; [3] primitives whose last energy balance did not converge. */
int hrt_last_stats(const hrt_context *ctx, uint64_t *stats, int count);
/* Device status word (HRT error bits) accumulated since the last reset. */
int hrt_device_status(hrt_context *ctx, uint32_t *status, int reset);

/* ---- inspection (tests): closest/any hit for explicit rays, the ray set of one
 * pass, and the device-built BVH (same layout as the host build). */
int hrt_trace_rays(hrt_context *ctx, int64_t nrays, const float *origins, const float *dirs, float tmin, float tmax,
                   int anyhit, int32_t *hit, float *t, int32_t *face);
int hrt_gen_rays(hrt_context *ctx, int kind, uint32_t seed, uint32_t pass, int32_t rays_per_primitive, int32_t face,
                 const float *direction, float *origins, float *dirs);
int hrt_get_bvh(hrt_context *ctx, uint64_t *codes, uint32_t *perm, uint32_t *nodes);
/* Measurement controls (no counterpart in the reference; used by the benchmark).
 * flags bit 0: run the statistics variants of the trace kernels, which count BVH
 * node visits and primitive tests (of the tree the default kernels traverse; with bit 2
 * also set, of the binary tree); bit 1: time every trace-kernel launch with CUDA
 * events on the context's stream.  Setting flags also resets the accumulators.
 * hrt_get_measure: [0] direct launches, [1] direct ms, [2] diffuse launches,
 * [3] diffuse ms, [4] node visits, [5] primitive tests, [6] rays of direct launches,
 * [7] rays of diffuse launches, [8] node visits and [9] primitive tests of diffuse launches
 * ([6]-[9] with bit 0, which syncs after every launch). */
int hrt_set_measure(hrt_context *ctx, int flags);
int hrt_get_measure(hrt_context *ctx, double *out, int count);
/* ---- BVH build that allocates nothing (no counterpart in the reference).
 * For callers that cannot call cudaMalloc -- code that hands out all device memory
 * from its own arena or framework allocator, and latency-critical loops where an
 * allocation would synchronise the device.  Builds the same LBVH as hrt_build_accel()
 * from caller-owned DEVICE buffers into caller-owned DEVICE buffers:
 *   d_transform [n*16] float, d_type [n] uint32 (inputs);
 *   d_records [n*64 B], d_origins [n*64 B], d_nodes [max(n-1,1)*64 B], d_codes [n],
 *   d_perm [n] (outputs; nodes/codes/perm in the hrt_get_bvh layout).
 * It takes no leaf area densities: voxels are built as empty boxes that no ray hits.
 * Scratch is a static device array sized for at most HRT_STATIC_MAX_PRIMS primitives
 * (about 5.6 MB held by every GPU that loads the library, until exit); larger n is
 * rejected with HRT_EINVAL.  The first call on a device looks the array's address up
 * and caches it per device index: make it before any stream capture, and reload the
 * library after a cudaDeviceReset of that device.  All calls share the array: calls
 * whose GPU work overlaps (other streams or threads) race.  Work is queued on
 * `stream` (a cudaStream_t, NULL = legacy default stream); the call then reads the
 * error word back and waits for that stream only (never the whole device) and returns
 * HRT_OK, HRT_EINVAL, HRT_ECUDA or HRT_EDEVICE (device error word set). */
#define HRT_STATIC_MAX_PRIMS 32768
int hrt_build_accel_static(const float *d_transform, const uint32_t *d_type, int32_t n, void *d_records,
                           void *d_origins, void *d_nodes, uint64_t *d_codes, uint32_t *d_perm, void *stream);
/* Rotation matrix (row-major 3x3) that rect/disk sources use, from Euler angles
 * (same convention as the reference's d_makeTransformMatrix, OptiX8DeviceCode.cu:191-201). */
void hrt_source_rotation(const float rotation[3], float out[9]);

#ifdef __cplusplus
}
#endif
#endif /* HRT_H */
