// dpx_amp.cpp — amplitude-grid files in D+'s binary format (version 13), so
// that grids computed here can be read by D+ and D+'s .amp files can be
// placed in a model (AmpGridAmplitude, Amplitude.cpp:3682-3720).
//
// Layout written by JacobianSphereGrid::ExportBinaryData (Grid.cpp:847-891)
// and read by ImportBinaryData (Grid.cpp:893-963):
//   "#@", uint32 offset of the data header (= 2 + 4 + 1 + len(header) + 1),
//   "\n", header text, "\n",
//   "13\n", "16\n" (bytes per complex double), "<L + 3>\n", "3\n",
//   the q step as a raw double, then 2 P doubles: the interleaved complex
//   amplitudes in grid-index order (no spline coefficients: the reader
//   recomputes them).
#include "dpx_host.h"

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

using namespace dpxh;

namespace {

constexpr unsigned kAmpVersion = 13;
constexpr int kExtras = 3;

struct File {
    FILE* f = nullptr;
    explicit File(FILE* p) : f(p) {}
    ~File() {
        if (f) std::fclose(f);
    }
};

// Reads one '\n'-terminated line (without the '\n'); false at end of file.
bool read_line(FILE* f, std::string& out) {
    out.clear();
    for (int c; (c = std::fgetc(f)) != EOF;) {
        if (c == '\n') return true;
        out.push_back((char)c);
    }
    return !out.empty();
}

// The header part of ImportBinaryData: descriptor, offset, '#' lines, then the
// numeric fields up to the raw q step.  Leaves f at the first data double.
int parse_header(FILE* f, int* grid_size, double* step, std::string& header) {
    unsigned offset = 0;
    int c = std::fgetc(f);
    if (c == '#') {
        const int c2 = std::fgetc(f);
        if (c2 == '@') {
            if (std::fread(&offset, sizeof offset, 1, f) != 1) return fail(DPX_ERR_ARG, "truncated .amp header");
            std::string del;
            read_line(f, del);
        } else if (c2 != '\n') {
            std::string line;
            read_line(f, line);
            header += std::string(1, (char)c2) + line + "\n";
        }
    } else if (c != EOF) {
        std::ungetc(c, f);
    }
    for (c = std::fgetc(f); c == '#'; c = std::fgetc(f)) {
        std::string line;
        read_line(f, line);
        header += "#" + line + "\n";
    }
    if (c != EOF) std::ungetc(c, f);
    if (offset > 0) {
        // the text between the descriptor and the offset is the header
        std::string text;
        if (std::fseek(f, 7, SEEK_SET) != 0) return fail(DPX_ERR_ARG, "bad .amp offset");
        for (long p = 7; p < (long)offset - 1; ++p) {
            const int ch = std::fgetc(f);
            if (ch == EOF) return fail(DPX_ERR_ARG, "truncated .amp header");
            text.push_back((char)ch);
        }
        header = text;
        if (std::fseek(f, (long)offset, SEEK_SET) != 0) return fail(DPX_ERR_ARG, "bad .amp offset");
    }
    unsigned version = 0, bytes = 0, dimx = 0, extras = 0;
    if (std::fscanf(f, "%u", &version) != 1) return fail(DPX_ERR_ARG, "no .amp version");
    if (version < 13) return fail(DPX_ERR_ARG, ".amp version %u is not a Jacobian sphere grid (13)", version);
    if (std::fscanf(f, "%u", &bytes) != 1 || bytes != 16) return fail(DPX_ERR_ARG, ".amp element size is not 16");
    if (std::fscanf(f, "%u", &dimx) != 1 || std::fscanf(f, "%u", &extras) != 1)
        return fail(DPX_ERR_ARG, "truncated .amp sizes");
    if ((int)extras != kExtras || dimx <= extras) return fail(DPX_ERR_ARG, "unsupported .amp grid extras");
    for (c = std::fgetc(f); c != '\n' && c != EOF; c = std::fgetc(f)) {
    }
    if (std::fread(step, sizeof(double), 1, f) != 1) return fail(DPX_ERR_ARG, "truncated .amp step");
    *grid_size = 2 * (int)(dimx - extras);
    return DPX_OK;
}

}  // namespace

extern "C" {

int dpx_amp_write(const char* path, const char* header, int grid_size, double step, const double* values) {
    if (!path || !values) return fail(DPX_ERR_ARG, "NULL argument");
    if (grid_size < 2 || (grid_size & 1)) return fail(DPX_ERR_ARG, "grid_size must be even and >= 2");
    const std::string head = header ? header : "";
    File out(std::fopen(path, "wb"));
    if (!out.f) return fail(DPX_ERR_ARG, "cannot open %s for writing", path);
    const unsigned headlen = (unsigned)(2 + sizeof(unsigned) + 1 + head.size() + 1);
    const int64_t P = dpx::make_geom(grid_size, 1.0).P;
    const std::string fields = std::to_string(kAmpVersion) + "\n16\n" + std::to_string(grid_size / 2 + kExtras) +
                               "\n" + std::to_string(kExtras) + "\n";
    bool ok = std::fwrite("#@", 1, 2, out.f) == 2 && std::fwrite(&headlen, sizeof headlen, 1, out.f) == 1;
    ok = ok && std::fputc('\n', out.f) != EOF && std::fwrite(head.data(), 1, head.size(), out.f) == head.size();
    ok = ok && std::fputc('\n', out.f) != EOF && std::fwrite(fields.data(), 1, fields.size(), out.f) == fields.size();
    ok = ok && std::fwrite(&step, sizeof step, 1, out.f) == 1;
    ok = ok && std::fwrite(values, sizeof(double), (size_t)(2 * P), out.f) == (size_t)(2 * P);
    if (!ok) return fail(DPX_ERR_ARG, "write to %s failed", path);
    return DPX_OK;
}

int dpx_amp_read_info(const char* path, int* grid_size, double* step, char* header, int64_t header_cap) {
    if (!path || !grid_size || !step) return fail(DPX_ERR_ARG, "NULL argument");
    File in(std::fopen(path, "rb"));
    if (!in.f) return fail(DPX_ERR_ARG, "cannot open %s", path);
    std::string head;
    if (int rc = parse_header(in.f, grid_size, step, head)) return rc;
    if (header && header_cap > 0) {
        const size_t n = std::min((size_t)header_cap - 1, head.size());
        std::memcpy(header, head.data(), n);
        header[n] = '\0';
    }
    return DPX_OK;
}

int dpx_amp_read(const char* path, double* values) {
    if (!path || !values) return fail(DPX_ERR_ARG, "NULL argument");
    File in(std::fopen(path, "rb"));
    if (!in.f) return fail(DPX_ERR_ARG, "cannot open %s", path);
    std::string head;
    int grid_size = 0;
    double step = 0;
    if (int rc = parse_header(in.f, &grid_size, &step, head)) return rc;
    const int64_t P = dpx::make_geom(grid_size, 1.0).P;
    if (std::fread(values, sizeof(double), (size_t)(2 * P), in.f) != (size_t)(2 * P))
        return fail(DPX_ERR_ARG, "%s holds fewer than %lld cells", path, (long long)P);
    return DPX_OK;
}

}  // extern "C"
