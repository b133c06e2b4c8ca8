// Oracle build support (test infrastructure only): a driver program over the
// reference's own simulation classes, built by oracle/ref/build_ref.py with
// the reference's CPU backend.  It runs the reference's VLM::run
// (vlm/src/vlm.cpp:97-151) and UVLM::run (vlm/src/vlm.cpp:358-509) and prints
// what they produce as JSON, so tests/golden/make_ref_golden.py can commit
// fixtures written by the reference's code rather than by the restatement.
//
//   ref_fixtures vlm  <alpha_deg,...> <mesh.x> [<mesh.x> ...]
//       per alpha: CL of VLM::run and every surface's circulation
//       (gamma_wing, column-major (ns, nc), i.e. chordwise row by row)
//   ref_fixtures mesh <mesh.x> <qc 0|1>
//       the vertices the reference's plot3d reader (MeshIO::read,
//       vlm/src/vlm_mesh.cpp:50-123) produces, x plane then y then z, each
//       column-major (ns+1, nc+1)
//   ref_fixtures uvlm <mesh.x> <t_final> <k> <heave_amp> <pitch_amp_deg> <pitch_phase_deg>
//       the reference's UVLM::run on a pitch-plunge motion: free stream
//       (-t, 0, 0), heave (0, 0, h sin(k t)) after it, pitch about the quarter
//       chord by a sin(k t + phase) after the heave; prints the time step and
//       the CL(t) record UVLM::run writes (cl_data_CPU.txt), and the final
//       circulation
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "vlm.hpp"
#include "vlm_kinematics.hpp"
#include "vlm_utils.hpp"

using namespace vlm;

static std::vector<float> parse_list(const char* s) {
    std::vector<float> out;
    std::stringstream ss(s);
    std::string item;
    while (std::getline(ss, item, ',')) out.push_back(std::stof(item));
    return out;
}

static void print_gamma(MultiTensor2fD& gamma) {
    std::printf("[");
    for (size_t m = 0; m < gamma.views().size(); m++) {
        const auto& g = gamma.views()[m];
        std::printf("%s[", m ? "," : "");
        for (i64 j = 0; j < g.shape(1); j++)
            for (i64 i = 0; i < g.shape(0); i++)
                std::printf("%s%.9g", (i || j) ? "," : "", (double)g(i, j));
        std::printf("]");
    }
    std::printf("]");
}

static int cmd_vlm(int argc, char** argv) {
    if (argc < 4) return 2;
    const std::vector<float> alphas = parse_list(argv[2]);
    std::vector<std::string> meshes;
    for (int i = 3; i < argc; i++) meshes.push_back(argv[i]);
    VLM sim{"cpu", meshes};
    std::printf("{\"cases\":[");
    for (size_t a = 0; a < alphas.size(); a++) {
        FlowData flow{to_radians(alphas[a]), 0.0f, 1.0f, 1.0f};
        const auto coeffs = sim.run(flow);
        std::printf("%s{\"alpha_deg\":%.9g,\"alpha\":%.9g,\"cl\":%.9g,\"gamma\":", a ? "," : "", (double)alphas[a],
                    (double)flow.alpha, (double)coeffs.cl);
        print_gamma(sim.gamma_wing);
        std::printf("}");
    }
    std::printf("]}\n");
    return 0;
}

static int cmd_uvlm(int argc, char** argv) {
    if (argc != 8) return 2;
    const std::string mesh = argv[2];
    const f32 t_final = std::stof(argv[3]);
    const f32 k = std::stof(argv[4]);
    const f32 h = std::stof(argv[5]);
    const f32 amp = to_radians(std::stof(argv[6]));
    const f32 phase = to_radians(std::stof(argv[7]));
    KinematicsTree<f32> tree;
    auto fs = tree.add([=](const fwd::Float& t) { return translation_matrix<fwd::Float>({-t, 0.f, 0.f}); });
    auto heave = tree.add([=](const fwd::Float& t) {
        return translation_matrix<fwd::Float>({0.f, 0.f, h * fwd::sin(k * t)});
    })->after(fs);
    auto pitch = tree.add([=](const fwd::Float& t) {
        return rotation_matrix<fwd::Float>({0.25f, 0.0f, 0.0f}, {0.0f, 1.0f, 0.0f}, amp * fwd::sin(phase + k * t));
    })->after(heave);
    Assembly<f32> assembly(fs);
    assembly.add(mesh, pitch);
    UVLM sim{"cpu", {mesh}};
    sim.run(assembly, t_final, k);
    // UVLM::run writes "<k>\n" then "t z cl angle" per step from the second on
    std::ifstream in("cl_data_" + sim.backend->name + ".txt");
    std::string line;
    std::getline(in, line);
    std::printf("{\"t\":[");
    std::vector<double> cols[4];
    double a, b, c, d;
    while (in >> a >> b >> c >> d) {
        cols[0].push_back(a);
        cols[1].push_back(b);
        cols[2].push_back(c);
        cols[3].push_back(d);
    }
    for (size_t i = 0; i < cols[0].size(); i++) std::printf("%s%.9g", i ? "," : "", cols[0][i]);
    std::printf("],\"z\":[");
    for (size_t i = 0; i < cols[1].size(); i++) std::printf("%s%.9g", i ? "," : "", cols[1][i]);
    std::printf("],\"cl\":[");
    for (size_t i = 0; i < cols[2].size(); i++) std::printf("%s%.9g", i ? "," : "", cols[2][i]);
    std::printf("],\"pitch\":[");
    for (size_t i = 0; i < cols[3].size(); i++) std::printf("%s%.9g", i ? "," : "", cols[3][i]);
    std::printf("],\"gamma_last\":");
    print_gamma(sim.gamma_wing);
    std::printf("}\n");
    return 0;
}

static int cmd_mesh(int argc, char** argv) {
    if (argc != 4) return 2;
    const MeshIO io{"plot3d"};
    const auto [nc, ns] = io.get_dims(argv[2]);
    Memory* mem = nullptr;
    std::vector<float> buf((size_t)(ns + 1) * (nc + 1) * 4, 1.0f);
    TensorView3fH v{mem, {ns + 1, nc + 1, 4}, {1, ns + 1, (ns + 1) * (nc + 1)}, buf.data()};
    io.read(argv[2], v, std::string(argv[3]) == "1");
    std::printf("{\"ns\":%lld,\"nc\":%lld,\"xyz\":[", (long long)ns, (long long)nc);
    for (i64 k = 0; k < 3; k++)
        for (i64 j = 0; j <= nc; j++)
            for (i64 i = 0; i <= ns; i++)
                std::printf("%s%.9g", (k || j || i) ? "," : "", (double)v(i, j, k));
    std::printf("]}\n");
    return 0;
}

int main(int argc, char** argv) {
    if (argc >= 2 && std::string(argv[1]) == "mesh") return cmd_mesh(argc, argv);
    if (argc >= 2 && std::string(argv[1]) == "vlm") return cmd_vlm(argc, argv);
    if (argc >= 2 && std::string(argv[1]) == "uvlm") return cmd_uvlm(argc, argv);
    std::fprintf(stderr, "usage: ref_fixtures vlm <alphas_deg> <mesh>...; ref_fixtures uvlm <mesh> <t_final> <k> "
                         "<heave> <pitch_deg> <phase_deg>\n");
    return 2;
}
