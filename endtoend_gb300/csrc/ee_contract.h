// ee_contract.h -- the temp-directory contract of the reference's
// dosecalc-preprocess, as its programs read it (host C++, header-only; shared
// by the dosecalc-beam and dosecalc-beamlet programs of this engine):
//   omni-header.txt       load_omni_header    (CCCS/DoseCalcIO/calc_header.cpp:81-136)
//   density.raw           load_density        (CCCS/DoseCalcIO/binary_io.cpp:13-32)
//   omni_beam_list.txt    load_omni_beam_list (CCCS/DoseCalcIO/beam.cpp:495-552)
//   fluence_maps/<file>   load_fluence_map    (CCCS/DoseCalcIO/fluence.cpp:19-43)
#pragma once
#include <sys/stat.h>
#include <unistd.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "ee_cccs.h"

namespace contract {

constexpr float kPi = 3.14159265358979323846f;
inline const char* program_name = "dosecalc";

struct Header {  // CONSTANTS fields of the omni-header (brain_defs.h:14-57)
    unsigned size[3] = {0, 0, 0};
    float voxel[3] = {0, 0, 0}, start[3] = {0, 0, 0};
    unsigned bbox_start[3] = {0, 0, 0}, bbox_size[3] = {0, 0, 0}, max_rev[3] = {0, 0, 0};
    float latspacing = 0, longspacing = 0, kernel_extent = 0, penumbra = 0;
    unsigned ss_factor = 1;
    int nphi = 0, ntheta = 0, nradii = 0, beam_count = 0, reduce = 0;
    std::string beam_spec, target_structure;
};

struct Beam {
    ee_beam b;
    std::string fmap_fname;
    std::vector<float> fluence;
};


inline int fail(const char* what, const std::string& detail = "") {
    std::fprintf(stderr, "%s: %s%s%s\n", program_name, what, detail.empty() ? "" : ": ", detail.c_str());
    return 1;
}

inline bool flag(const char* arg, const char* name, std::string* value) {
    const size_t n = std::strlen(name);
    if (std::strncmp(arg, "--", 2) != 0 || std::strncmp(arg + 2, name, n) != 0) return false;
    const char* rest = arg + 2 + n;
    if (*rest == '\0') {
        if (value) value->clear();
        return true;
    }
    if (*rest != '=') return false;
    if (value) *value = rest + 1;
    return true;
}

inline void chomp(char* s) {
    size_t n = std::strlen(s);
    while (n > 0 && (s[n - 1] == '\n' || s[n - 1] == '\r')) s[--n] = '\0';
}

// omni-header: comment lines start with '#' or ' '; the first other line
// (the blank separator) is consumed, then the fields follow in order.
inline int load_header(const std::string& path, Header& H) {
    FILE* f = std::fopen(path.c_str(), "r");
    if (!f) return fail("cannot open the omni-header", path);
    char line[1024];
    for (;;) {
        if (!std::fgets(line, sizeof(line), f)) {
            std::fclose(f);
            return fail("omni-header ends inside its comment block", path);
        }
        if (line[0] != '#' && line[0] != ' ') break;
    }
    int ok = 0;
    ok += std::fscanf(f, "%u %u %u", &H.size[0], &H.size[1], &H.size[2]);
    ok += std::fscanf(f, "%f %f %f", &H.voxel[0], &H.voxel[1], &H.voxel[2]);
    ok += std::fscanf(f, "%f %f %f", &H.start[0], &H.start[1], &H.start[2]);
    ok += std::fscanf(f, "%u %u %u", &H.bbox_start[0], &H.bbox_start[1], &H.bbox_start[2]);
    ok += std::fscanf(f, "%u %u %u", &H.bbox_size[0], &H.bbox_size[1], &H.bbox_size[2]);
    ok += std::fscanf(f, "%u %u %u", &H.max_rev[0], &H.max_rev[1], &H.max_rev[2]);
    ok += std::fscanf(f, "%f", &H.latspacing);
    ok += std::fscanf(f, "%f", &H.longspacing);
    ok += std::fscanf(f, "%f", &H.kernel_extent);
    ok += std::fscanf(f, "%u", &H.ss_factor);
    ok += std::fscanf(f, "%d %d %d", &H.nphi, &H.ntheta, &H.nradii);
    ok += std::fscanf(f, "%f", &H.penumbra);
    ok += std::fscanf(f, "%d", &H.beam_count);
    char spec[1024] = {0}, target[1024] = {0};
    bool lines = std::fgets(line, sizeof(line), f) && std::fgets(spec, sizeof(spec), f) &&
                 std::fgets(target, sizeof(target), f);
    ok += std::fscanf(f, "%d", &H.reduce);
    std::fclose(f);
    if (ok != 28 || !lines) return fail("malformed omni-header", path);
    chomp(spec);
    chomp(target);
    H.beam_spec = spec;
    H.target_structure = target;
    // a valid calc bbox, as load_omni_header enforces (calc_header.cpp:127-133)
    for (int a = 0; a < 3; a++) {
        if (H.bbox_start[a] >= H.size[a]) H.bbox_start[a] = 0;
        if (H.bbox_size[a] + H.bbox_start[a] > H.size[a]) H.bbox_size[a] = H.size[a] - H.bbox_start[a];
    }
    return 0;
}

inline int read_floats(const std::string& path, size_t n, std::vector<float>& out) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return fail("cannot open", path);
    out.resize(n);
    const size_t got = std::fread(out.data(), sizeof(float), n, f);
    std::fclose(f);
    if (got != n) return fail("file shorter than expected", path + " (" + std::to_string(got) + " of " +
                                                               std::to_string(n) + " floats)");
    return 0;
}

// omni_beam_list.txt: a count, then one 22-field record per beam; angles in
// degrees, converted with the reference's FP32 (deg * pi) / 180.
inline int load_beams(const std::string& temp, int header_count, std::vector<Beam>& beams) {
    const std::string path = temp + "/omni_beam_list.txt";
    FILE* f = std::fopen(path.c_str(), "r");
    if (!f) return fail("cannot open the beam list", path);
    int count = 0;
    if (std::fscanf(f, "%d", &count) != 1 || count < 0) {
        std::fclose(f);
        return fail("malformed beam list", path);
    }
    if (header_count < count) count = header_count;
    beams.resize(count > 0 ? count : 0);
    for (int b = 0; b < count; b++) {
        int id = 0;
        char iso_type[32], iso_loc[32], orient[32], fname[1024];
        float az, zen, coll, sad, iso[3], src[3], dir[3], bl[2];
        int fm[2];
        const int n = std::fscanf(f, " %d %f %f %f %f %31s %31s %f %f %f %f %f %f %31s %f %f %f %f %f %d %d %1023s", &id,
                                  &az, &zen, &coll, &sad, iso_type, iso_loc, &iso[0], &iso[1], &iso[2], &src[0],
                                  &src[1], &src[2], orient, &dir[0], &dir[1], &dir[2], &bl[0], &bl[1], &fm[0], &fm[1],
                                  fname);
        if (n != 22) {
            std::fclose(f);
            return fail("malformed beam record", path + " record " + std::to_string(b + 1));
        }
        Beam& B = beams[b];
        B.b.azimuth = (az * kPi) / 180.0f;
        B.b.zenith = (zen * kPi) / 180.0f;
        B.b.coll = (coll * kPi) / 180.0f;
        for (int a = 0; a < 3; a++) B.b.isocenter[a] = iso[a];
        B.b.sad = sad;
        B.b.fmap_size[0] = fm[0];
        B.b.fmap_size[1] = fm[1];
        B.b.beamlet_size[0] = bl[0];
        B.b.beamlet_size[1] = bl[1];
        B.fmap_fname = fname;
        if (fm[0] <= 0 || fm[1] <= 0) {
            std::fclose(f);
            return fail("beam record with an empty fluence map", path);
        }
    }
    std::fclose(f);
    for (Beam& B : beams)
        if (read_floats(temp + "/fluence_maps/" + B.fmap_fname, (size_t)B.b.fmap_size[0] * B.b.fmap_size[1],
                        B.fluence))
            return 1;
    return 0;
}

inline bool exists(const std::string& p) {
    struct stat st;
    return ::stat(p.c_str(), &st) == 0;
}

inline int mkdirs(const std::string& dir) {
    if (dir.empty() || exists(dir)) return 0;
    const size_t slash = dir.find_last_of('/');
    if (slash != std::string::npos && slash > 0) mkdirs(dir.substr(0, slash));
    return ::mkdir(dir.c_str(), 0755) == 0 || exists(dir) ? 0 : 1;
}

inline int check(int st, const char* what) {
    if (st == EE_OK) return 0;
    return fail(what, ee_last_error());
}

}  // namespace contract
