// Run-time check of the C++ boundary: reads a cloud (n, then xyz, normals as float32 and
// rgb as uint8, each n x 3), builds the reference's 64-byte DepthSurfel records on the
// device, reconstructs through the shim's SolvePoissionReconstructionMesh(const
// DepthSurfel*, int) and writes the mesh (vertex count, triangle count, vertices,
// triangles, colours, normals).  Then it serves the same cloud twice through the
// header-only Server (two slots, host inputs and outputs) and checks both meshes equal
// the shim's.  Usage: shim_main cloud.bin mesh.bin
#include <cstdio>
#include <cstring>
#include <vector>

#include "psr/PoissonReconstruction.hpp"
#include "psr/Server.hpp"

int main(int argc, char** argv) {
    if (argc < 3) return 2;
    FILE* f = fopen(argv[1], "rb");
    if (!f) return 3;
    int n = 0;
    if (fread(&n, 4, 1, f) != 1) return 3;
    std::vector<float> xyz(3 * (size_t)n), nrm(3 * (size_t)n);
    std::vector<unsigned char> rgb(3 * (size_t)n);
    if (fread(xyz.data(), 4, xyz.size(), f) != xyz.size() || fread(nrm.data(), 4, nrm.size(), f) != nrm.size() ||
        fread(rgb.data(), 1, rgb.size(), f) != rgb.size())
        return 3;
    fclose(f);
    std::vector<psr_gb300::DepthSurfel> surf((size_t)n);
    for (int i = 0; i < n; ++i) {
        psr_gb300::DepthSurfel& s = surf[i];
        s.row = s.col = 0;
        s.VertexAndConfidence = make_float4(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], 1.0f);
        s.NormalAndRadius = make_float4(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2], 0.0f);
        s.ColorAndTime = make_float4(rgb[3 * i] / 255.0f, rgb[3 * i + 1] / 255.0f, rgb[3 * i + 2] / 255.0f, 0.0f);
    }
    psr_gb300::DepthSurfel* d_surf = nullptr;
    if (cudaMalloc(&d_surf, sizeof(psr_gb300::DepthSurfel) * (size_t)n) != cudaSuccess) return 4;
    cudaMemcpy(d_surf, surf.data(), sizeof(psr_gb300::DepthSurfel) * (size_t)n, cudaMemcpyHostToDevice);
    psr_config cfg;
    psr_config_default(&cfg);
    cfg.max_depth = 7;
    cfg.max_points = n;
    cfg.compute_colors = 1;
    cfg.compute_normals = 1;
    psr_gb300::PoissonReconstruction recon(&cfg);
    recon.SolvePoissionReconstructionMesh(d_surf, n);
    const auto& V = recon.GetRebuildMeshVertices();
    const auto& T = recon.GetRebuildMeshTriangleIndices();
    const auto& C = recon.GetRebuildMeshColors();
    const auto& N = recon.GetRebuildMeshNormals();
    FILE* o = fopen(argv[2], "wb");
    const int nv = (int)V.size(), nt = (int)T.size();
    fwrite(&nv, 4, 1, o);
    fwrite(&nt, 4, 1, o);
    fwrite(V.data(), 12, V.size(), o);
    fwrite(T.data(), 12, T.size(), o);
    fwrite(C.data(), 12, C.size(), o);
    fwrite(N.data(), 12, N.size(), o);
    fclose(o);
    // the same cloud twice through the served form
    psr_gb300::Server srv(cfg, 2);
    std::vector<float> sv[2], sc[2], sn[2];
    std::vector<int> st[2];
    psr_mesh mesh[2];
    psr_gb300::Server::Request req[2];
    for (int k = 0; k < 2; ++k) {
        sv[k].resize(3 * (size_t)cfg.max_mesh_vertices);
        sc[k].resize(3 * (size_t)cfg.max_mesh_vertices);
        sn[k].resize(3 * (size_t)cfg.max_mesh_vertices);
        st[k].resize(3 * (size_t)cfg.max_triangles);
        memset(&mesh[k], 0, sizeof(psr_mesh));
        mesh[k].vertices = sv[k].data();
        mesh[k].triangles = st[k].data();
        mesh[k].colors = sc[k].data();
        mesh[k].normals = sn[k].data();
        mesh[k].vertex_capacity = cfg.max_mesh_vertices;
        mesh[k].triangle_capacity = cfg.max_triangles;
        mesh[k].location = PSR_HOST;
        req[k].points = psr_points{xyz.data(), nrm.data(), rgb.data(), n, PSR_HOST};
        req[k].options = psr_options{7, 0};
        req[k].mesh = &mesh[k];
        srv.submit(&req[k]);
    }
    while (srv.step() || srv.queued()) {
    }
    for (int k = 0; k < 2; ++k) {
        if (req[k].status != PSR_OK) { printf("served %d: status %d\n", k, (int)req[k].status); return 5; }
        if (mesh[k].vertex_count != nv || mesh[k].triangle_count != nt ||
            memcmp(sv[k].data(), V.data(), 12 * (size_t)nv) || memcmp(st[k].data(), T.data(), 12 * (size_t)nt) ||
            memcmp(sc[k].data(), C.data(), 12 * (size_t)nv) || memcmp(sn[k].data(), N.data(), 12 * (size_t)nv)) {
            printf("served %d: mesh differs from the shim's\n", k);
            return 6;
        }
    }
    printf("ok %d vertices %d triangles, served twice identically (%d slots)\n", nv, nt, srv.slots());
    cudaFree(d_surf);
    return 0;
}
