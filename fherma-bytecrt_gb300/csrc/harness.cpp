// `solution <point dir>`: runs every case of a point directory through the
// plugin ABI and records what each call cost.  Same wire format as the
// challenge's generated harness (native-smoke/main.cpp:1-17, :106-133):
//
//   <dir>/manifest.json           {"N":..,"W":..,"L":..,"cases":..} (+ "B" when batched)
//   <dir>/point/q.bin             L little-endian uint32
//   <dir>/cases/NNNNNN/{a,b}.bin  [N][L] (or [B][N][L]) uint32
//   <dir>/out/NNNNNN/c.bin        written
//   <dir>/out/results.json        {"init_s":..,"cases":[{"i":..,"seconds":..,"status":"ok"}, ...]}
//
// Only fherma_run is timed (steady clock).  A case that throws is recorded as
// "crashed" with a note and the run continues; results.json is rewritten
// after every case so a killed run keeps what it finished.
#include "fherma.h"

#include <chrono>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <iostream>
#include <sstream>
#include <vector>

namespace fs = std::filesystem;

namespace {

std::string read_file(const fs::path& p) {
    std::ifstream f(p, std::ios::binary);
    if (!f) throw std::runtime_error("cannot open " + p.string());
    std::stringstream ss;
    ss << f.rdbuf();
    return ss.str();
}

double manifest_number(const std::string& text, const char* key, bool required = true) {
    const std::string needle = std::string("\"") + key + "\"";
    const size_t at = text.find(needle);
    if (at == std::string::npos) {
        if (required) throw std::runtime_error(std::string("manifest.json lacks ") + key);
        return -1;
    }
    const size_t colon = text.find(':', at + needle.size());
    return std::strtod(text.c_str() + colon + 1, nullptr);
}

fherma::Tensor<uint32_t> read_tensor(const fs::path& file, std::vector<int64_t> shape) {
    fherma::Tensor<uint32_t> t;
    t.shape = std::move(shape);
    const std::string raw = read_file(file);
    const size_t n = size_t(t.count());
    if (raw.size() != n * 4)
        throw std::runtime_error(file.filename().string() + ": " + std::to_string(raw.size()) + " bytes, want " +
                                 std::to_string(n * 4));
    t.data.resize(n);
    std::memcpy(t.data.data(), raw.data(), raw.size());
    return t;
}

std::string case_name(size_t i) {
    char buf[32];
    std::snprintf(buf, sizeof buf, "%06zu", i);
    return buf;
}

std::string json_escape(const std::string& s) {
    std::string out;
    for (char ch : s.substr(0, 200)) {
        if (ch == '"' || ch == '\\') out += '\\';
        out += (ch == '\n') ? ' ' : ch;
    }
    return out;
}

void write_results(const fs::path& out, double init_s, const std::vector<std::string>& rows) {
    std::ofstream f(out / "results.json");
    char head[64];
    std::snprintf(head, sizeof head, "{\"init_s\":%.9f,\"cases\":[", init_s);
    f << head;
    for (size_t i = 0; i < rows.size(); ++i) f << (i ? "," : "") << rows[i];
    f << "]}";
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) {
        std::cerr << "usage: solution <point directory>\n";
        return 2;
    }
    const fs::path root = argv[1];
    const std::string manifest = read_file(root / "manifest.json");
    fherma::Point p;
#ifdef FHERMA_BATCHED
    p.B = uint32_t(manifest_number(manifest, "B"));
#endif
    p.N = uint32_t(manifest_number(manifest, "N"));
    p.W = uint32_t(manifest_number(manifest, "W"));
    p.L = uint32_t(manifest_number(manifest, "L"));
    p.q = read_tensor(root / "point" / "q.bin", {int64_t(p.L)});
    const size_t cases = size_t(manifest_number(manifest, "cases"));
    std::vector<int64_t> shape = {int64_t(p.N), int64_t(p.L)};
#ifdef FHERMA_BATCHED
    shape.insert(shape.begin(), int64_t(p.B));
#endif
    const fs::path out_root = root / "out";
    fs::create_directories(out_root);

    const auto t0 = std::chrono::steady_clock::now();
    void* state = fherma_init(p);
    const double init_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::vector<std::string> rows;
    write_results(out_root, init_s, rows);

    for (size_t i = 0; i < cases; ++i) {
        const fs::path dir = root / "cases" / case_name(i);
        char row[256];
        fherma::Inputs in;
        try {
            in.a = read_tensor(dir / "a.bin", shape);
            in.b = read_tensor(dir / "b.bin", shape);
        } catch (const std::exception& e) {
            rows.push_back("{\"i\":" + std::to_string(i) + ",\"seconds\":null,\"status\":\"crashed\",\"note\":\"" +
                           json_escape(std::string("reading the case: ") + e.what()) + "\"}");
            write_results(out_root, init_s, rows);
            continue;
        }
        fherma::Outputs answer;
        double seconds = 0;
        try {
            const auto s = std::chrono::steady_clock::now();
            answer = fherma_run(state, in);
            seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - s).count();
        } catch (const std::exception& e) {
            rows.push_back("{\"i\":" + std::to_string(i) + ",\"seconds\":null,\"status\":\"crashed\",\"note\":\"" +
                           json_escape(e.what()) + "\"}");
            write_results(out_root, init_s, rows);
            continue;
        }
        try {
            fs::create_directories(out_root / case_name(i));
            std::ofstream f(out_root / case_name(i) / "c.bin", std::ios::binary);
            f.write(reinterpret_cast<const char*>(answer.c.data.data()), std::streamsize(answer.c.data.size() * 4));
            if (!f) throw std::runtime_error("short write of c.bin");
        } catch (const std::exception& e) {
            rows.push_back("{\"i\":" + std::to_string(i) + ",\"seconds\":null,\"status\":\"crashed\",\"note\":\"" +
                           json_escape(std::string("writing the answer: ") + e.what()) + "\"}");
            write_results(out_root, init_s, rows);
            continue;
        }
        std::snprintf(row, sizeof row, "{\"i\":%zu,\"seconds\":%.9f,\"status\":\"ok\"}", i, seconds);
        rows.push_back(row);
        write_results(out_root, init_s, rows);
    }
    fherma_free(state);
    write_results(out_root, init_s, rows);
    return 0;
}
