// Header-only C++ shim over the C ABI (psr.h) with the reference's class and method names
// (SparseSurfelFusion::PoissonReconstruction, mesh/PoissonReconstruction.h:63-184), so a
// caller of the reference's data-parallel path can switch by changing the include and the
// namespace.  Besides the handle it owns one device buffer, allocated in the constructor
// for max_points surfels, into which the DepthSurfel overload unpacks the surfels; no
// reconstruction call allocates.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <stdexcept>
#include <string>
#include <vector>

#include "psr.h"

namespace psr_gb300 {

// Layout of the reference's DepthSurfel (base/CommonTypes.h:113-118): 8-byte pixel
// coordinate, then position+confidence, normal+radius and colour+time as float4.
struct DepthSurfel {
    unsigned int row, col;
    float4 VertexAndConfidence;
    float4 NormalAndRadius;
    float4 ColorAndTime;
};
static_assert(sizeof(DepthSurfel) == 64, "DepthSurfel must keep the reference's 64-byte layout");

struct Point3D {
    float coords[3];
};
struct TriangleIndex {
    int idx[3];
};

class PoissonReconstruction {
public:
    explicit PoissonReconstruction(const psr_config* cfg = nullptr) {
        psr_config c;
        if (cfg) c = *cfg;
        else psr_config_default(&c);
        cfg_ = c;
        psr_status s = psr_create(&c, &h_);
        if (s != PSR_OK) throw std::runtime_error(std::string("psr_create: ") + psr_status_string(s));
        // SoA staging of the DepthSurfel overload: xyz, normals (floats) and rgb (bytes)
        cudaError_t e = cudaMalloc(&staging_, 6 * sizeof(float) * (size_t)c.max_points + 3 * (size_t)c.max_points);
        if (e != cudaSuccess) {
            psr_destroy(h_);
            h_ = nullptr;
            throw std::runtime_error(std::string("surfel staging: ") + cudaGetErrorString(e));
        }
        staging_count_ = c.max_points;
    }
    ~PoissonReconstruction() {
        if (h_) psr_destroy(h_);
        if (staging_) cudaFree(staging_);
    }
    PoissonReconstruction(const PoissonReconstruction&) = delete;
    PoissonReconstruction& operator=(const PoissonReconstruction&) = delete;

    // Same role as the reference's SolvePoissionReconstructionMesh(DeviceArrayView<DepthSurfel>):
    // device-resident surfels in, mesh kept in the object (read with the getters below).
    void SolvePoissionReconstructionMesh(const DepthSurfel* device_surfels, int count, cudaStream_t stream = nullptr) {
        if (count > staging_count_) throw std::runtime_error("more surfels than max_points");
        float* xyz = staging_;
        float* nrm = staging_ + 3 * (size_t)count;
        // colour from ColorAndTime.xyz when the handle transfers colours
        uint8_t* rgb = cfg_.compute_colors ? (uint8_t*)(staging_ + 6 * (size_t)count) : nullptr;
        psr_status s = psr_surfels_to_points(device_surfels, count, xyz, nrm, rgb, stream);
        if (s != PSR_OK) throw std::runtime_error(std::string("psr_surfels_to_points: ") + psr_status_string(s));
        Solve(xyz, nrm, rgb, count, PSR_DEVICE, stream);
    }

    // Oriented points (host or device), optional 8-bit colour.
    void Solve(const float* xyz, const float* normals, const uint8_t* rgb, int count, int location,
               cudaStream_t stream = nullptr, int depth = 0, int cg_iterations = 0) {
        vertices_.resize((size_t)cfg_.max_mesh_vertices);
        triangles_.resize((size_t)cfg_.max_triangles);
        colors_.resize(cfg_.compute_colors ? (size_t)cfg_.max_mesh_vertices : 0);
        normals_.resize(cfg_.compute_normals ? (size_t)cfg_.max_mesh_vertices : 0);
        psr_points p{xyz, normals, rgb, count, location};
        psr_options o{depth, cg_iterations};
        psr_mesh m{};
        m.vertices = (float*)vertices_.data();
        m.triangles = (int32_t*)triangles_.data();
        m.colors = cfg_.compute_colors ? (float*)colors_.data() : nullptr;
        m.normals = cfg_.compute_normals ? (float*)normals_.data() : nullptr;
        m.vertex_capacity = cfg_.max_mesh_vertices;
        m.triangle_capacity = cfg_.max_triangles;
        m.location = PSR_HOST;
        psr_status s = psr_reconstruct(h_, &p, &o, &m, stream);
        if (s != PSR_OK)
            throw std::runtime_error(std::string("psr_reconstruct: ") + psr_status_string(s) + ": " + psr_last_error(h_));
        vertices_.resize((size_t)m.vertex_count);
        triangles_.resize((size_t)m.triangle_count);
        if (cfg_.compute_colors) colors_.resize((size_t)m.vertex_count);
        if (cfg_.compute_normals) normals_.resize((size_t)m.vertex_count);
        center_[0] = m.center[0]; center_[1] = m.center[1]; center_[2] = m.center[2];
        scale_ = m.scale;
    }

    // Normals of an unoriented cloud (the reference's PCL step, CalculatePointCloudNormal,
    // mesh/PoissonReconstruction.cpp:137-161: k = 10, viewpoint at the origin by default);
    // xyz and normals are 3 * count floats in `location` memory.  NaN for clouds of fewer
    // than 3 points.
    void CalculatePointCloudNormal(const float* xyz, int count, float* normals, int location = PSR_HOST,
                                   const float* viewpoint = nullptr, cudaStream_t stream = nullptr) {
        psr_status s = psr_estimate_normals(h_, xyz, count, (psr_location)location, normals, viewpoint, stream);
        if (s != PSR_OK)
            throw std::runtime_error(std::string("psr_estimate_normals: ") + psr_status_string(s) + ": " +
                                     psr_last_error(h_));
    }

    // Unoriented host points: normals estimated on the GPU, then the reconstruction (the
    // reference's readPCDFile followed by SolvePoissionReconstructionMesh)
    void SolveUnoriented(const float* xyz, int count, const uint8_t* rgb = nullptr) {
        std::vector<float> nrm(3 * (size_t)count);
        CalculatePointCloudNormal(xyz, count, nrm.data(), PSR_HOST);
        // no normal (NaN: degenerate neighbourhood) -> zero, which adds nothing to the field
        for (size_t i = 0; i < nrm.size(); i += 3)
            if (!(std::isfinite(nrm[i]) && std::isfinite(nrm[i + 1]) && std::isfinite(nrm[i + 2])))
                nrm[i] = nrm[i + 1] = nrm[i + 2] = 0.0f;
        Solve(xyz, nrm.data(), rgb, count, PSR_HOST);
    }

    // mesh/ComputeTriangleIndices.h:331-342 (host copies here)
    const std::vector<Point3D>& GetRebuildMeshVertices() const { return vertices_; }
    const std::vector<TriangleIndex>& GetRebuildMeshTriangleIndices() const { return triangles_; }
    const std::vector<Point3D>& GetRebuildMeshColors() const { return colors_; }
    const std::vector<Point3D>& GetRebuildMeshNormals() const { return normals_; }
    const float* BoundingBoxOrigin() const { return center_; }
    float BoundingBoxEdge() const { return scale_; }
    psr_handle* handle() const { return h_; }

private:
    psr_config cfg_{};
    psr_handle* h_ = nullptr;
    float* staging_ = nullptr;
    int staging_count_ = 0;
    std::vector<Point3D> vertices_;
    std::vector<TriangleIndex> triangles_;
    std::vector<Point3D> colors_;
    std::vector<Point3D> normals_;
    float center_[3] = {0, 0, 0};
    float scale_ = 0;
};

}  // namespace psr_gb300
