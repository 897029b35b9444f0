// adapter_runband.cpp -- drives the C++ drop-in adapter (helios::GB300Backend) through
// RadiationModel::runBand's sequence of backend calls (plugins/radiation/src/
// RadiationModel.cpp:3779-4356 and 4628-4663) and writes the per-primitive flux.
//
//   adapter_runband <input bundle> <output flux file>
//
// The input bundle (written by tests/test_gpu_backend_adapter.py) is a list of named arrays:
// name '\0', kind byte ('f' float32, 'i' int32, 'u' uint32, 'b' byte), uint64 count, data.
// The output is n * Bl float32 values, [primitive][launched band].
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "GB300Backend.h"

namespace {

struct Blob {
    char kind = 0;
    uint64_t count = 0;
    std::vector<char> bytes;
};

std::map<std::string, Blob> read_bundle(const char *path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error(std::string("cannot open ") + path);
    std::map<std::string, Blob> out;
    for (;;) {
        std::string name;
        char c;
        while (f.get(c) && c != '\0') name.push_back(c);
        if (!f) break;
        Blob b;
        f.get(b.kind);
        f.read(reinterpret_cast<char *>(&b.count), sizeof b.count);
        const size_t esz = b.kind == 'b' ? 1 : 4;
        b.bytes.resize(b.count * esz);
        f.read(b.bytes.data(), (std::streamsize)b.bytes.size());
        if (!f) throw std::runtime_error("truncated bundle at " + name);
        out[name] = std::move(b);
    }
    return out;
}

template <class T>
std::vector<T> arr(const std::map<std::string, Blob> &m, const char *name) {
    auto it = m.find(name);
    if (it == m.end()) throw std::runtime_error(std::string("missing array ") + name);
    std::vector<T> v(it->second.bytes.size() / sizeof(T));
    std::memcpy(v.data(), it->second.bytes.data(), v.size() * sizeof(T));
    return v;
}

template <class T>
T maxof(const std::vector<T> &v) {
    T m = v.empty() ? T(0) : v[0];
    for (const T &x : v) m = x > m ? x : m;
    return m;
}

}  // namespace

int main(int argc, char **argv) {
    if (argc != 3) {
        std::cerr << "usage: adapter_runband <bundle> <flux out>\n";
        return 2;
    }
    try {
        const auto in = read_bundle(argv[1]);
        const auto T = arr<float>(in, "T");
        const auto type = arr<uint32_t>(in, "type");
        const auto ts = arr<int8_t>(in, "twosided");
        const auto bbox = arr<float>(in, "bbox");
        const auto periodic = arr<float>(in, "periodic");
        const auto rho = arr<float>(in, "rho"), tau = arr<float>(in, "tau");
        const auto src = arr<float>(in, "sources");  // [S][type, pos3, width2, rot3]
        const auto src_flux = arr<float>(in, "source_flux");
        const auto band_launch = arr<uint8_t>(in, "band_launch");
        const auto depth = arr<int32_t>(in, "depth");
        const auto direct_rays = arr<int32_t>(in, "direct_rays"), diffuse_rays = arr<int32_t>(in, "diffuse_rays");
        const auto emission = arr<uint8_t>(in, "emission");
        const auto eps = arr<float>(in, "eps");
        const auto temperature = arr<float>(in, "temperature");
        const auto diffuse_flux = arr<float>(in, "diffuse_flux");
        const auto dext = arr<float>(in, "diffuse_ext"), dnorm = arr<float>(in, "diffuse_norm");
        const auto dpeak = arr<float>(in, "diffuse_peak"), prague = arr<float>(in, "prague");
        const uint32_t seed = arr<uint32_t>(in, "seed").at(0);

        const size_t n = type.size();
        const size_t S = src.size() / 9;
        const size_t Bg = band_launch.size();
        size_t Bl = 0;
        for (uint8_t f : band_launch) Bl += f ? 1 : 0;

        helios::RayTracingGeometry geom;
        geom.primitive_count = n;
        geom.transform_matrices = T;
        geom.primitive_types.assign(type.begin(), type.end());
        geom.twosided_flags.assign(ts.begin(), ts.end());
        geom.bbox_count = bbox.size() / 12;
        for (size_t k = 0; k + 2 < bbox.size(); k += 3) geom.bboxes.vertices.push_back({bbox[k], bbox[k + 1], bbox[k + 2]});
        geom.bboxes.count = geom.bbox_count;
        geom.periodic_flag = {periodic.at(0), periodic.at(1)};

        helios::RayTracingMaterial mat;
        mat.num_sources = S;
        mat.num_primitives = n;
        mat.num_bands = Bg;
        mat.reflectivity = rho;
        mat.transmissivity = tau;

        std::vector<helios::RayTracingSource> sources(S);
        for (size_t s = 0; s < S; ++s) {
            const float *q = &src[9 * s];
            sources[s].type = (uint)q[0];
            sources[s].position = {q[1], q[2], q[3]};
            sources[s].width = {q[4], q[5]};
            sources[s].rotation = {q[6], q[7], q[8]};
        }

        // RadiationModel::updateGeometry / updateRadiativeProperties (RadiationModel.cpp:1981-1982, 2916)
        helios::GB300Backend be(0);
        be.initialize();
        be.updateGeometry(geom);
        be.buildAccelerationStructure();
        be.updateMaterials(mat);
        be.updateSources(sources);

        bool scattering = false, diffuse = false, any_emission = false, rundirect = false;
        for (int32_t d : depth) scattering = scattering || d > 0;
        for (float f : diffuse_flux) diffuse = diffuse || f > 0.f;
        for (uint8_t e : emission) any_emission = any_emission || e;
        for (float f : src_flux) rundirect = rundirect || f > 0.f;
        const uint32_t dirN = (uint32_t)maxof(direct_rays), difN = (uint32_t)maxof(diffuse_rays);
        const int dmax = maxof(depth);

        auto base = [&](const std::vector<uint8_t> &flags) {
            helios::RayTracingLaunchParams p;
            p.launch_offset = 0;
            p.launch_count = (uint)n;
            p.random_seed = seed;
            p.num_bands_global = (uint)Bg;
            p.num_bands_launch = (uint)Bl;
            p.band_launch_flag.assign(flags.begin(), flags.end());
            for (size_t b = 0; b < Bl; ++b) {
                p.diffuse_extinction.push_back(dext[b]);
                p.diffuse_dist_norm.push_back(dnorm[b]);
                p.diffuse_peak_dir.push_back({dpeak[3 * b], dpeak[3 * b + 1], dpeak[3 * b + 2]});
                p.sky_radiance_params.push_back({prague[4 * b], prague[4 * b + 1], prague[4 * b + 2], prague[4 * b + 3]});
            }
            return p;
        };

        be.zeroRadiationBuffers(Bl);                                   // :3804
        be.uploadSourceFluxes(src_flux);                               // :3822
        if (S > 0 && rundirect) {                                      // :3927
            auto p = base(band_launch);
            p.rays_per_primitive = dirN;
            be.launchDirectRays(p);
        }
        std::vector<float> ftop(n * Bl, 0.f), fbot(n * Bl, 0.f);
        helios::RayTracingResults res;
        if (scattering && rundirect) {                                 // :3999-4037, one-sided fold
            be.getRadiationResults(res);
            ftop = res.scatter_buff_top;
            fbot = res.scatter_buff_bottom;
            for (size_t p = 0; p < n; ++p)
                if (ts[p] == 0)
                    for (size_t b = 0; b < Bl; ++b) {
                        const float t = ftop[p * Bl + b] + fbot[p * Bl + b];
                        ftop[p * Bl + b] = fbot[p * Bl + b] = t;
                    }
            be.uploadRadiationOut(ftop, fbot);
            be.zeroScatterBuffers();
        }
        const uint32_t side = (uint32_t)std::ceil(std::sqrt((double)difN));
        const uint32_t rpp = side * side;
        const float sigma = 5.6703744e-8f;  // RadiationModel.h:2210
        if (any_emission || diffuse) {
            if (any_emission) {                                        // :4041-4137
                for (size_t b = 0; b < Bl; ++b) {
                    if (!emission[b]) continue;
                    for (size_t p = 0; p < n; ++p) {
                        float e = eps[p * Bl + b];
                        if (depth[b] == 0 && e != 1.f) e = 1.f;
                        const double Tk = (double)temperature[p];
                        const float out = (float)((double)(sigma * e) * (Tk * Tk * Tk * Tk));
                        ftop[p * Bl + b] += out;
                        if (ts[p] != 0) fbot[p * Bl + b] += out;
                    }
                }
            }
            for (uint32_t face : {1u, 0u}) {                            // :4161-4209
                auto p = base(band_launch);
                p.rays_per_primitive = rpp;
                p.scattering_iteration = 0;
                p.launch_face = face;
                p.diffuse_flux = diffuse_flux;
                p.radiation_out_top = ftop;
                p.radiation_out_bottom = fbot;
                be.launchDiffuseRays(p);
            }
        }
        if (scattering && (any_emission || diffuse) && !rundirect) {
            be.copyScatterToRadiation();
            be.zeroScatterBuffers();
        }
        if (scattering && (any_emission || diffuse || rundirect)) {    // :4236-4356
            std::vector<uint8_t> sflags = band_launch;
            const std::vector<float> zero(Bl, 0.f);
            for (int it = 0; it < dmax; ++it) {
                int b = -1;
                for (size_t bg = 0; bg < Bg; ++bg) {
                    if (!sflags[bg]) continue;
                    ++b;
                    if (it + 1 > depth[(size_t)b]) sflags[bg] = 0;     // launched-band compaction
                }
                if (it > 0 || (any_emission && rundirect)) be.copyScatterToRadiation();
                be.zeroScatterBuffers();
                be.getRadiationResults(res);
                for (uint32_t face : {1u, 0u}) {
                    auto p = base(sflags);
                    p.rays_per_primitive = rpp;
                    p.scattering_iteration = (uint)(it + 1);
                    p.launch_face = face;
                    p.diffuse_flux = zero;
                    p.radiation_out_top = res.radiation_out_top;
                    p.radiation_out_bottom = res.radiation_out_bottom;
                    be.launchDiffuseRays(p);
                }
            }
        }
        be.getRadiationResults(res);                                   // :4628-4663
        std::vector<float> flux(n * Bl);
        for (size_t i = 0; i < n * Bl; ++i)
            flux[i] = res.radiation_in[i] + res.scatter_buff_top[i] + res.scatter_buff_bottom[i];
        std::ofstream o(argv[2], std::ios::binary);
        o.write(reinterpret_cast<const char *>(flux.data()), (std::streamsize)(flux.size() * sizeof(float)));
        std::cout << "backend " << be.getBackendName() << ": " << n << " primitives, " << Bl << " bands\n";
        be.shutdown();
        return o ? 0 : 1;
    } catch (const std::exception &e) {
        std::cerr << "adapter_runband: " << e.what() << "\n";
        return 1;
    }
}
