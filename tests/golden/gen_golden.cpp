// Golden-vector generator for the parity tests.
//
// Restates the population generators and the host-side expectation code of
// the reference's own tests (libstdc++'s std::mt19937_64 default-seeded and
// std::uniform_*_distribution, exactly as those tests draw them), and writes
// inputs + expected outputs as raw little-endian arrays. make_golden.py runs
// this and packs the arrays into .npz fixtures. The expectations are computed
// here the way the reference tests compute them (bin counts summed over the
// Moore neighbourhood), independently of the oracle's PBM code.
//
//   tests/test_cases/runtime/messaging/test_spatial_3d.cu:72-200  (Mandatory)
//   tests/test_cases/runtime/messaging/test_spatial_3d.cu:248-330 (Optional)
//   tests/test_cases/runtime/messaging/test_spatial_2d.cu:66-185  (Mandatory)
//   tests/test_cases/runtime/messaging/test_spatial_2d.cu:186-320 (Optional)
//   tests/test_cases/simulation/test_cuda_simulation.cu:406-434   (AgentDeath)
#include <cstdio>
#include <cstdint>
#include <random>
#include <string>
#include <unordered_map>
#include <vector>

static void dump(const std::string& dir, const std::string& name, const void* p, size_t bytes) {
    FILE* f = std::fopen((dir + "/" + name).c_str(), "wb");
    if (!f) { std::perror(name.c_str()); std::exit(1); }
    std::fwrite(p, 1, bytes, f);
    std::fclose(f);
}

// Moore-neighbourhood expectation over a D-dimensional grid of edge E.
static unsigned expected3(std::unordered_map<int, unsigned>& bc, int E, unsigned x1, unsigned y1, unsigned z1) {
    unsigned s = 0;
    for (int a = -1; a <= 1; ++a)
        for (int b = -1; b <= 1; ++b)
            for (int c = -1; c <= 1; ++c) {
                const int p[3] = {static_cast<int>(x1) + a, static_cast<int>(y1) + b, static_cast<int>(z1) + c};
                if (p[0] >= 0 && p[1] >= 0 && p[2] >= 0 && p[0] < E && p[1] < E && p[2] < E)
                    s += bc[p[2] * E * E + p[1] * E + p[0]];
            }
    return s;
}
static unsigned expected2(std::unordered_map<int, unsigned>& bc, int E, unsigned x1, unsigned y1) {
    unsigned s = 0;
    for (int a = -1; a <= 1; ++a)
        for (int b = -1; b <= 1; ++b) {
            const int p[2] = {static_cast<int>(x1) + a, static_cast<int>(y1) + b};
            if (p[0] >= 0 && p[1] >= 0 && p[0] < E && p[1] < E) s += bc[p[1] * E + p[0]];
        }
    return s;
}

static void spatial3d(const std::string& dir, bool optional) {
    const int N = 2049, E = 5;
    std::mt19937_64 rng;
    std::uniform_real_distribution<float> dist(0.0f, 5.0f);
    std::vector<float> pos(3 * N);
    std::vector<int32_t> do_output(N, 1);
    std::vector<uint32_t> mybin(N), expect(N);
    std::unordered_map<int, unsigned> bc, bco;
    for (int i = 0; i < N; ++i) {
        float p[3] = {dist(rng), dist(rng), dist(rng)};
        if (optional) do_output[i] = dist(rng) < 4 ? 1 : 0;
        for (int a = 0; a < 3; ++a) pos[3 * i + a] = p[a];
        const unsigned bp[3] = {(unsigned)(p[0] / 1), (unsigned)(p[1] / 1), (unsigned)(p[2] / 1)};
        mybin[i] = bp[2] * E * E + bp[1] * E + bp[0];
        bc[mybin[i]] += 1;
        if (do_output[i]) bco[mybin[i]] += 1;
    }
    for (int i = 0; i < N; ++i) {
        const unsigned b = mybin[i];
        expect[i] = expected3(optional ? bco : bc, E, b % E, (b / E) % E, b / (E * E));
    }
    const std::string pre = optional ? "s3d_optional_" : "s3d_mandatory_";
    dump(dir, pre + "pos.f32", pos.data(), pos.size() * 4);
    dump(dir, pre + "do_output.i32", do_output.data(), N * 4);
    dump(dir, pre + "mybin.u32", mybin.data(), N * 4);
    dump(dir, pre + "expect.u32", expect.data(), N * 4);
}

static void spatial2d(const std::string& dir, bool optional) {
    const int N = 2049, E = 11;
    std::mt19937_64 rng;
    std::uniform_real_distribution<float> dist(0.0f, 11.0f);
    std::uniform_real_distribution<float> dist5(0.0f, 5.0f);
    std::vector<float> pos(2 * N);
    std::vector<int32_t> do_output(N, 1);
    std::vector<uint32_t> mybin(N), expect(N);
    std::unordered_map<int, unsigned> bc, bco;
    for (int i = 0; i < N; ++i) {
        float p[3] = {dist(rng), dist(rng), dist(rng)};  // the reference test draws 3 per agent
        if (optional) do_output[i] = dist5(rng) < 4 ? 1 : 0;
        pos[2 * i] = p[0];
        pos[2 * i + 1] = p[1];
        const unsigned bp[2] = {(unsigned)(p[0] / 1), (unsigned)(p[1] / 1)};
        mybin[i] = bp[1] * E + bp[0];
        bc[mybin[i]] += 1;
        if (do_output[i]) bco[mybin[i]] += 1;
    }
    for (int i = 0; i < N; ++i) {
        const unsigned b = mybin[i];
        expect[i] = expected2(optional ? bco : bc, E, b % E, b / E);
    }
    const std::string pre = optional ? "s2d_optional_" : "s2d_mandatory_";
    dump(dir, pre + "pos.f32", pos.data(), pos.size() * 4);
    dump(dir, pre + "do_output.i32", do_output.data(), N * 4);
    dump(dir, pre + "mybin.u32", mybin.data(), N * 4);
    dump(dir, pre + "expect.u32", expect.data(), N * 4);
}

static void agent_death(const std::string& dir) {
    const int N = 10;
    std::mt19937_64 generator;
    std::uniform_int_distribution<unsigned int> distribution(0, 12);
    std::vector<uint32_t> x(N), expect;
    for (int i = 0; i < N; ++i) {
        x[i] = distribution(generator);
        if (x[i] % 2 != 0) expect.push_back(x[i]);
    }
    dump(dir, "death_x.u32", x.data(), N * 4);
    dump(dir, "death_expect.u32", expect.data(), expect.size() * 4);
}

int main(int argc, char** argv) {
    if (argc < 2) { std::fprintf(stderr, "usage: gen_golden <outdir>\n"); return 2; }
    const std::string dir = argv[1];
    spatial3d(dir, false);
    spatial3d(dir, true);
    spatial2d(dir, false);
    spatial2d(dir, true);
    agent_death(dir);
    return 0;
}
