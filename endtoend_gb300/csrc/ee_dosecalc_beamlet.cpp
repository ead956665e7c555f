// ee_dosecalc_beamlet.cpp -- `dosecalc-beamlet`, the reference's beamlet
// dose-coefficient program (CCCS/dosecalc-beamlet/main.cu), on the GB300
// engine through the ee_* C ABI only.
//
// Inputs: the same temp-dir contract as dosecalc-beam (ee_contract.h), the
// header's kernel_extent and REV size limits, and the spectrum and dsa point
// kernels under $data (the cumulative kernel is rebuilt by
// ee_cumulative_kernel, bit-identical to cumulative_kernel.h5).  Every beamlet
// with positive fluence gets a sparse dose column; entries are kept where
// value > thresh * column max (CCCS/DoseCalcIO/sparse_io.cpp:22-59), default
// threshold 1e-6 as the reference's (main.cu:48).
//
// Output: Dose_Coefficients.h5 (doc/schema_doc/beamlet_data_output.md) needs
// HDF5, which is not available here.  The same per-beam datasets are written
// as raw little-endian files in the directory <dir of --out>/<stem of --out>/
// (default ./Dose_Coefficients/):
//   calc_specs.txt                 the calc_specs attributes, "key value" lines
//   beam_NNNNN.txt                 the beam's metadata, "key value" lines
//   beam_NNNNN_beamlet_index.raw   int32  [N_beamlets]  fluence-map index of each column
//   beam_NNNNN_col_ptr.raw         int64  [N_beamlets+1]
//   beam_NNNNN_lindex.raw          uint32 [nnz]  full-grid voxel index, x fastest, ascending per column
//   beam_NNNNN_coeffs.raw          float32 [nnz]
//
// ROI reduction (the header's `reduce` flag, as main.cu:293-308 and
// sparse_io.cpp:160-172): the reference reads the ROI masks from
// <temp>/roi_list.h5, which needs HDF5.  Here they come from
// <temp>/roi_list.txt (or --roi-list=FILE): one ROI per line,
//   name x0 y0 z0 nx ny nz mask_file
// mask_file (relative to the list's directory) holds the crop box's
// nx*ny*nz uint8 flags, x fastest.  With ROIs, every column is reduced by
// ee_roi_reduce and the coefficient files become
//   beam_NNNNN_lindex.raw          uint64 [nnz]  row within the ROI row blocks
//   beam_NNNNN_row_blocks.raw      int64  [N_beamlets][N_rois]  rows kept per ROI
// and calc_specs.txt gains roi_order and row_block_capacities.  Without a
// list the columns are written unreduced, as the reference does when it
// finds no ROI file.
#include <chrono>
#include <cstdio>
#include <string>
#include <vector>

#include "ee_contract.h"

using namespace contract;

namespace {

struct Options {
    std::string out = "./Dose_Coefficients.h5", temp, data, roi_list;
    float thresh = 1e-6f;
    int device = 0, ndevices = 1;
    bool verbose = false, timing = false, dry_run = false;
};

void usage() {
    std::printf(
        "dosecalc-beamlet (GB300 engine): sparse beamlet dose coefficients from the dosecalc-preprocess\n"
        "temp directory.\n\n"
        "Usage:  dosecalc-beamlet [options...]\n"
        " Optional Args:\n"
        "  --out=[outfile]                  result name; the coefficients go to the directory <stem>/ beside it\n"
        "                                   (default ./Dose_Coefficients/)\n"
        "  --ndevices=[<int>]               accepted; the engine runs every beam on one GPU\n"
        "  --device=[<int>]                 GPU to use\n"
        "  --sparsify-threshold=[<float>]   keep value > threshold * column max [default: 1.00e-06]\n"
        "  --roi-list=[<file>]              ROI masks for the row reduction (default <temp>/roi_list.txt when\n"
        "                                   the header requests a reduction)\n"
        "                                   (also --thresh, --sparsity-threshold)\n"
        "  --temp=[<dir>]                   temp directory (default /tmp/dosecalc/$USER)\n"
        "  --data=[<dir>]                   data directory with spectra/ and dsa/ (default $DOSECALC_DATA or ./data)\n"
        "  --dry-run                        read and check every input, print a summary, no GPU work\n"
        "  --verbose                        output calculation progress information\n"
        "  --timing                         output calculation timing information\n"
        "  --help                           show this help message\n");
}

double now_ms() {
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

template <class T>
int write_raw(const std::string& path, const std::vector<T>& v) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) return fail("cannot open the output file", path);
    const size_t put = v.empty() ? 0 : std::fwrite(v.data(), sizeof(T), v.size(), f);
    std::fclose(f);
    if (put != v.size()) return fail("short write", path);
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    program_name = "dosecalc-beamlet";
    Options O;
    {
        const char* user = std::getenv("USER");
        O.temp = std::string("/tmp/dosecalc/") + (user && *user ? user : "unknown");
        const char* d = std::getenv("DOSECALC_DATA");
        O.data = d && *d ? d : "./data";
    }
    for (int i = 1; i < argc; i++) {
        std::string v;
        const char* a = argv[i];
        if (flag(a, "help", nullptr)) {
            usage();
            return 0;
        } else if (flag(a, "out", &v)) O.out = v;
        else if (flag(a, "device", &v)) O.device = std::atoi(v.c_str());
        else if (flag(a, "ndevices", &v)) O.ndevices = std::atoi(v.c_str());
        else if (flag(a, "sparsify-threshold", &v) || flag(a, "thresh", &v) || flag(a, "sparsity-threshold", &v)) {
            char* end = nullptr;
            O.thresh = std::strtof(v.c_str(), &end);
            if (v.empty() || *end != '\0' || !(O.thresh >= 0.f)) return fail("bad sparsify threshold", v);
        } else if (flag(a, "temp", &v)) O.temp = v;
        else if (flag(a, "roi-list", &v)) O.roi_list = v;
        else if (flag(a, "data", &v)) O.data = v;
        else if (flag(a, "dry-run", nullptr)) O.dry_run = true;
        else if (flag(a, "verbose-extra", nullptr) || flag(a, "verbose", nullptr)) O.verbose = true;
        else if (flag(a, "timing", nullptr)) O.timing = true;
        else if (flag(a, "srworkers", nullptr) || flag(a, "debug", nullptr) || flag(a, "debug-extra", nullptr) ||
                 std::strncmp(a, "--srworkers=", 12) == 0) {
        } else {
            usage();
            return fail("unknown argument", a);
        }
    }
    const double t0 = now_ms();

    // ---- inputs (as dosecalc-beam)
    Header H;
    if (load_header(O.temp + "/omni-header.txt", H)) return 1;
    if (H.nradii != EE_DSA_NRADII) return fail("nradii must be 24 (the dsa kernels)", std::to_string(H.nradii));
    const size_t nvox = (size_t)H.size[0] * H.size[1] * H.size[2];
    std::vector<float> density;
    if (read_floats(O.temp + "/density.raw", nvox, density)) return 1;
    std::vector<Beam> beams;
    if (load_beams(O.temp, H.beam_count, beams)) return 1;
    if (beams.empty()) return fail("no beams in the beam list");
    float energy[64], fluence[64], mu[64], mu_en[64];
    char names[64 * 256];
    int nE = 0;
    const std::string spec = O.data + "/spectra/" + H.beam_spec + ".spec";
    if (check(ee_read_spectrum_file(spec.c_str(), 64, energy, fluence, mu, mu_en, names, 256, &nE),
              "reading the spectrum"))
        return 1;
    const size_t cells = (size_t)EE_DSA_NCATEGORIES * EE_DSA_NANGLES * EE_DSA_NRADII;
    std::vector<float> mono((size_t)nE * cells);
    for (int e = 0; e < nE; e++) {
        const std::string k = O.data + "/dsa/" + std::string(names + 256 * e);
        if (check(ee_read_mono_kernel(k.c_str(), mono.data() + e * cells), "reading a point kernel")) return 1;
    }
    float radii[EE_DSA_NRADII];
    if (check(ee_read_kernel_radii((O.data + "/dsa/radii.dat").c_str(), radii), "reading radii.dat")) return 1;
    const int nrays = H.nphi * (H.ntheta / 2);
    std::vector<float> theta(nrays > 0 ? nrays : 1), phi(nrays > 0 ? nrays : 1);
    const std::string tf = O.temp + "/convolution_theta_angles.raw", pf = O.temp + "/convolution_phi_angles.raw";
    const bool angle_files = exists(tf) && exists(pf);
    if (angle_files && (read_floats(tf, nrays, theta) || read_floats(pf, nrays, phi))) return 1;
    // ---- ROI masks for the row reduction
    std::string roi_path = O.roi_list;
    if (roi_path.empty() && H.reduce) {
        if (exists(O.temp + "/roi_list.txt")) roi_path = O.temp + "/roi_list.txt";
        else if (exists(O.temp + "/roi_list.h5"))
            std::printf("note: %s/roi_list.h5 needs HDF5, which is not available; give the masks as roi_list.txt "
                        "(see --help); columns are written unreduced\n", O.temp.c_str());
    }
    std::vector<std::string> roi_names;
    std::vector<std::vector<unsigned char>> roi_bytes;
    std::vector<ee_roi_mask> roi_masks;
    if (!roi_path.empty()) {
        FILE* rf = std::fopen(roi_path.c_str(), "r");
        if (!rf) return fail("cannot open the ROI list", roi_path);
        const size_t sl = roi_path.find_last_of('/');
        const std::string rdir = sl == std::string::npos ? "." : roi_path.substr(0, sl);
        char line[4096];
        while (std::fgets(line, sizeof(line), rf)) {
            char name[1024], file[2048];
            int c0[3], cn[3];
            if (line[0] == '#') continue;
            const int got = std::sscanf(line, "%1023s %d %d %d %d %d %d %2047s", name, &c0[0], &c0[1], &c0[2], &cn[0],
                                        &cn[1], &cn[2], file);
            if (got <= 0) continue;
            if (got != 8 || cn[0] <= 0 || cn[1] <= 0 || cn[2] <= 0) {
                std::fclose(rf);
                return fail("malformed ROI list line", line);
            }
            std::vector<unsigned char> m((size_t)cn[0] * cn[1] * cn[2]);
            const std::string mp = file[0] == '/' ? std::string(file) : rdir + "/" + file;
            FILE* mf = std::fopen(mp.c_str(), "rb");
            const size_t got_b = mf ? std::fread(m.data(), 1, m.size(), mf) : 0;
            if (mf) std::fclose(mf);
            if (got_b != m.size()) {
                std::fclose(rf);
                return fail("ROI mask file missing or short", mp);
            }
            roi_names.push_back(name);
            roi_bytes.push_back(std::move(m));
            ee_roi_mask rm;
            for (int a = 0; a < 3; a++) {
                rm.crop_start[a] = c0[a];
                rm.crop_size[a] = cn[a];
            }
            rm.mask = nullptr;
            roi_masks.push_back(rm);
        }
        std::fclose(rf);
        for (size_t r = 0; r < roi_masks.size(); r++) roi_masks[r].mask = roi_bytes[r].data();
        if (roi_masks.empty()) return fail("no ROI in the list", roi_path);
    }
    ee_roi_list* rois = nullptr;
    std::vector<long long> capacities(roi_masks.size());
    if (!roi_masks.empty()) {
        const int vsize[3] = {(int)H.size[0], (int)H.size[1], (int)H.size[2]};
        if (check(ee_roi_list_create(vsize, roi_masks.data(), (int)roi_masks.size(), &rois), "reading the ROI masks") ||
            check(ee_roi_list_capacities(rois, capacities.data()), "reading the ROI masks"))
            return 1;
    }
    long long active = 0;
    for (const Beam& B : beams)
        for (float v : B.fluence) active += v > 0.f;
    const double t_read = now_ms();
    if (O.verbose || O.dry_run)
        std::printf("omni-header: size %u %u %u, bbox %u %u %u + %u %u %u, nphi %d ntheta %d, kernel_extent %g cm, "
                    "max_rev %u %u %u, spectrum %s; %zu beams, %lld beamlets with fluence, threshold %g\n",
                    H.size[0], H.size[1], H.size[2], H.bbox_start[0], H.bbox_start[1], H.bbox_start[2],
                    H.bbox_size[0], H.bbox_size[1], H.bbox_size[2], H.nphi, H.ntheta, H.kernel_extent, H.max_rev[0],
                    H.max_rev[1], H.max_rev[2], H.beam_spec.c_str(), beams.size(), active, O.thresh);
    if ((O.verbose || O.dry_run) && rois)
        std::printf("ROI reduction: %zu ROIs from %s\n", roi_masks.size(), roi_path.c_str());
    if (O.dry_run) {
        ee_roi_list_destroy(rois);
        std::printf("dry run: inputs read in %.1f ms\n", t_read - t0);
        return 0;
    }

    // ---- output directory
    std::string dir = ".", stem = O.out;
    const size_t slash = O.out.find_last_of('/');
    if (slash != std::string::npos) {
        dir = O.out.substr(0, slash);
        stem = O.out.substr(slash + 1);
    }
    const size_t dot = stem.find_last_of('.');
    if (dot != std::string::npos && dot > 0) stem = stem.substr(0, dot);
    const std::string odir = dir + "/" + stem;
    if (mkdirs(odir)) return fail("cannot create the output directory", odir);

    // ---- engine
    std::vector<float> cum((size_t)H.ntheta * EE_DSA_NRADII), th_k(theta.size()), ph_k(phi.size());
    if (check(ee_cumulative_kernel(O.device, nE, energy, fluence, mu, mono.data(), H.ntheta, H.nphi, cum.data(),
                                   nullptr, nullptr, nullptr, th_k.data(), ph_k.data()),
              "building the cumulative kernel"))
        return 1;
    if (!angle_files) {
        theta = th_k;
        phi = ph_k;
    }
    ee_context* ctx = nullptr;
    if (check(ee_create(O.device, &ctx), "creating the engine context")) return 1;
    int rc = 0;
    long long total_nnz = 0, total_cols = 0;
    double t_set = now_ms(), t_cols = 0;
    do {
        ee_frame fr;
        for (int a = 0; a < 3; a++) {
            fr.size[a] = (int)H.size[a];
            fr.voxel[a] = H.voxel[a];
            fr.start[a] = H.start[a];
            fr.bbox_start[a] = (int)H.bbox_start[a];
            fr.bbox_size[a] = (int)H.bbox_size[a];
        }
        if ((rc = check(ee_set_volume(ctx, &fr, density.data()), "setting the volume"))) break;
        if ((rc = check(ee_set_spectrum(ctx, nE, energy, fluence, mu, mu_en), "setting the spectrum"))) break;
        ee_conv_params cp = {H.ntheta, H.nphi, H.nradii, H.latspacing, H.longspacing, H.penumbra, {0, 0, 0}};
        if ((rc = check(ee_set_kernel_table(ctx, &cp, radii, cum.data(), theta.data(), phi.data()),
                        "setting the kernel table")))
            break;
        // REV size limits of the header (0: the engine's default, 500 per axis)
        int max_rev[3] = {500, 500, 500};
        for (int a = 0; a < 3; a++)
            if (H.max_rev[a] > 0) max_rev[a] = (int)H.max_rev[a];
        if ((rc = check(ee_set_beamlet_options(ctx, H.kernel_extent, max_rev), "setting the beamlet options"))) break;
        t_set = now_ms();
        for (size_t b = 0; b < beams.size() && !rc; b++) {
            ee_csr csr;
            if ((rc = check(ee_beamlet_columns_device(ctx, &beams[b].b, beams[b].fluence.data(), O.thresh, &csr),
                            "computing the beamlet columns")))
                break;
            std::vector<int> bidx(csr.nbeamlets);
            std::vector<long long> cptr(csr.nbeamlets + 1);
            std::vector<unsigned> lidx(csr.nnz);
            std::vector<float> coef(csr.nnz);
            if (csr.nbeamlets > 0 &&
                ((rc = check(ee_copy_to_host(ctx, bidx.data(), csr.beamlet_index, sizeof(int) * bidx.size()),
                             "reading the columns")) ||
                 (rc = check(ee_copy_to_host(ctx, cptr.data(), csr.col_ptr, sizeof(long long) * cptr.size()),
                             "reading the columns"))))
                break;
            if (csr.nbeamlets == 0) cptr[0] = 0;
            if (csr.nnz > 0 &&
                ((rc = check(ee_copy_to_host(ctx, lidx.data(), csr.row_index, sizeof(unsigned) * lidx.size()),
                             "reading the columns")) ||
                 (rc = check(ee_copy_to_host(ctx, coef.data(), csr.value, sizeof(float) * coef.size()),
                             "reading the columns"))))
                break;
            char base[64];
            std::snprintf(base, sizeof(base), "/beam_%05zu", b);
            const std::string pre = odir + base;
            long long nnz_out = csr.nnz;
            if (rois) {  // _sparsify_and_reduce: the sparsified column, then the ROI rows
                const size_t nr = roi_masks.size();
                std::vector<unsigned long long> rkeys;
                std::vector<float> rvals;
                std::vector<long long> rptr(1, 0), blocks((size_t)csr.nbeamlets * nr);
                for (int c = 0; c < csr.nbeamlets && !rc; c++) {
                    const long long a0 = cptr[c], n = cptr[c + 1] - cptr[c];
                    const size_t at = rkeys.size();
                    rkeys.resize(at + (size_t)n * nr);
                    rvals.resize(at + (size_t)n * nr);
                    long long got = 0;
                    rc = check(ee_roi_reduce(rois, reinterpret_cast<const int*>(lidx.data()) + a0, coef.data() + a0, n,
                                             rkeys.data() + at, rvals.data() + at, n * (long long)nr, &got,
                                             blocks.data() + (size_t)c * nr),
                               "reducing a column to the ROIs");
                    rkeys.resize(at + (size_t)got);
                    rvals.resize(at + (size_t)got);
                    rptr.push_back((long long)rkeys.size());
                }
                if (rc) break;
                nnz_out = (long long)rkeys.size();
                if ((rc = write_raw(pre + "_beamlet_index.raw", bidx)) || (rc = write_raw(pre + "_col_ptr.raw", rptr)) ||
                    (rc = write_raw(pre + "_lindex.raw", rkeys)) || (rc = write_raw(pre + "_coeffs.raw", rvals)) ||
                    (rc = write_raw(pre + "_row_blocks.raw", blocks)))
                    break;
            } else if ((rc = write_raw(pre + "_beamlet_index.raw", bidx)) ||
                       (rc = write_raw(pre + "_col_ptr.raw", cptr)) || (rc = write_raw(pre + "_lindex.raw", lidx)) ||
                       (rc = write_raw(pre + "_coeffs.raw", coef)))
                break;
            FILE* m = std::fopen((pre + ".txt").c_str(), "w");
            if (!m) {
                rc = fail("cannot open the output file", pre + ".txt");
                break;
            }
            const ee_beam& e = beams[b].b;
            std::fprintf(m, "beam_uid %zu\nN_beamlets %d\nN_coeffs %lld\ngantry_rot_rad %.9g\ncouch_rot_rad %.9g\n"
                            "coll_rot_rad %.9g\niso_coords_cm %.9g %.9g %.9g\nsad_cm %.9g\nfmap_size %d %d\n"
                            "beamlet_size_cm %.9g %.9g\nfmap_file %s\n",
                         b, csr.nbeamlets, nnz_out, e.azimuth, e.zenith, e.coll, e.isocenter[0], e.isocenter[1],
                         e.isocenter[2], e.sad, e.fmap_size[0], e.fmap_size[1], e.beamlet_size[0], e.beamlet_size[1],
                         beams[b].fmap_fname.c_str());
            std::fclose(m);
            total_nnz += nnz_out;
            total_cols += csr.nbeamlets;
            if (O.verbose) std::printf("beam %zu: %d columns, %lld coefficients\n", b, csr.nbeamlets, csr.nnz);
        }
        t_cols = now_ms();
    } while (false);
    ee_destroy(ctx);
    ee_roi_list_destroy(rois);
    if (rc) return rc;
    FILE* f = std::fopen((odir + "/calc_specs.txt").c_str(), "w");
    if (!f) return fail("cannot open the output file", odir + "/calc_specs.txt");
    std::fprintf(f, "N_beams %zu\ncalc_bbox_start %u %u %u\ncalc_bbox_size %u %u %u\npenumbra_cm %.9g\nconvlat_cm %.9g\n"
                    "convstep_cm %.9g\ndicom_start_cm %.9g %.9g %.9g\nfull_dicom_size %u %u %u\nnphi %d\nnradii %d\n"
                    "ntheta %d\nsparsity_thresh %.9g\nvoxel_size_cm %.9g %.9g %.9g\nkernel_extent_cm %.9g\n"
                    "beam_spectrum %s\ntarget_structure %s\n",
                 beams.size(), H.bbox_start[0], H.bbox_start[1], H.bbox_start[2], H.bbox_size[0], H.bbox_size[1],
                 H.bbox_size[2], H.penumbra, H.latspacing, H.longspacing, H.start[0], H.start[1], H.start[2],
                 H.size[0], H.size[1], H.size[2], H.nphi, H.nradii, H.ntheta, O.thresh, H.voxel[0], H.voxel[1],
                 H.voxel[2], H.kernel_extent, H.beam_spec.c_str(), H.target_structure.c_str());
    if (!roi_names.empty()) {
        std::fprintf(f, "roi_order");
        for (const auto& n : roi_names) std::fprintf(f, " %s", n.c_str());
        std::fprintf(f, "\nrow_block_capacities");
        for (long long c : capacities) std::fprintf(f, " %lld", c);
        std::fprintf(f, "\n");
    }
    std::fclose(f);
    std::printf("Data written to \"%s/\" (%zu beams, %lld columns, %lld coefficients); Dose_Coefficients.h5 not "
                "written (no HDF5 library)\n",
                odir.c_str(), beams.size(), total_cols, total_nnz);
    if (O.timing)
        std::printf("timing [ms]: read inputs %.1f, kernel + set-up %.1f, columns %.1f, total %.1f\n", t_read - t0,
                    t_set - t_read, t_cols - t_set, now_ms() - t0);
    return 0;
}
