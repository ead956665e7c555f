// ee_dosecalc_beam.cpp -- `dosecalc-beam`, the command-line program of the
// reference (CCCS/dosecalc-beam/main.cu), on the GB300 engine through the
// ee_* C ABI only.
//
// It reads the temp-dir contract that dosecalc-preprocess writes and writes
// the summed dose:
//   $temp/omni-header.txt         load_omni_header   (DoseCalcIO/calc_header.cpp:81-136)
//   $temp/density.raw             load_density       (DoseCalcIO/binary_io.cpp:13-32)
//   $temp/omni_beam_list.txt      load_omni_beam_list (DoseCalcIO/beam.cpp:495-552)
//   $temp/fluence_maps/<file>     load_fluence_map   (DoseCalcIO/fluence.cpp:19-43)
//   $temp/convolution_{theta,phi}_angles.raw  (DoseCalcIO/kernel.cpp:449-464)
//   $data/spectra/<beam_spec>.spec, $data/dsa/*      the spectrum (main.cu:188-203)
// $temp defaults to /tmp/dosecalc/$USER and $data to $DOSECALC_DATA or ./data,
// as Paths::Initialize does (DoseCalcIO/paths.cpp:6-20); --temp / --data
// override them.  The cumulative kernel of cumulative_kernel.h5 (HDF5, not
// available here) is rebuilt from the spectrum and the dsa point kernels by
// ee_cumulative_kernel, which reproduces make_cumulative_kernel bit for bit.
// Output: <dir of --out>/<stem of --out>.raw (default ./Dose.raw), FP32, x
// fastest, the full volume (main.cu:386-392).  Dose.h5 is not written.
#include <chrono>
#include <cstdio>
#include <string>
#include <vector>

#include "ee_contract.h"

using namespace contract;

namespace {

struct Options {
    std::string out = "./Dose.h5", temp, data, kernel = "table";
    int device = 0, ndevices = 1;
    bool verbose = false, timing = false, dry_run = false;
};

void usage() {
    std::printf(
        "dosecalc-beam (GB300 engine): full-beam dose from the dosecalc-preprocess temp directory.\n\n"
        "Usage:  dosecalc-beam [options...]\n"
        " Optional Args:\n"
        "  --out=[outfile]      result file; the dose is written beside it as <stem>.raw (default ./Dose.raw)\n"
        "  --ndevices=[<int>]   accepted; the engine batches every beam on one GPU\n"
        "  --device=[<int>]     GPU to use\n"
        "  --temp=[<dir>]       temp directory (default /tmp/dosecalc/$USER)\n"
        "  --data=[<dir>]       data directory with spectra/ and dsa/ (default $DOSECALC_DATA or ./data)\n"
        "  --kernel=table|exp   cumulative-table walk (the reference's, default) or the fitted\n"
        "                       double-exponential fast path\n"
        "  --dry-run            read and check every input, print a summary, no GPU work\n"
        "  --verbose            output calculation progress information\n"
        "  --timing             output calculation timing information\n"
        "  --help               show this help message\n");
}

double now_ms() {
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

}  // namespace

int main(int argc, char** argv) {
    program_name = "dosecalc-beam";
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
        else if (flag(a, "temp", &v)) O.temp = v;
        else if (flag(a, "data", &v)) O.data = v;
        else if (flag(a, "kernel", &v)) O.kernel = v;
        else if (flag(a, "dry-run", nullptr)) O.dry_run = true;
        else if (flag(a, "verbose-extra", nullptr) || flag(a, "verbose", nullptr)) O.verbose = true;
        else if (flag(a, "timing", nullptr)) O.timing = true;
        else if (flag(a, "debug", nullptr) || flag(a, "debug-extra", nullptr)) {
        } else {
            usage();
            return fail("unknown argument", a);
        }
    }
    if (O.kernel != "table" && O.kernel != "exp") return fail("--kernel must be table or exp", O.kernel);
    const double t0 = now_ms();

    // ---- inputs
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
    const double t_read = now_ms();
    if (O.verbose || O.dry_run) {
        std::printf("omni-header: size %u %u %u, voxel %g %g %g cm, bbox %u %u %u + %u %u %u, nphi %d ntheta %d, "
                    "ss_factor %u, spectrum %s (%d energies)\n",
                    H.size[0], H.size[1], H.size[2], H.voxel[0], H.voxel[1], H.voxel[2], H.bbox_start[0],
                    H.bbox_start[1], H.bbox_start[2], H.bbox_size[0], H.bbox_size[1], H.bbox_size[2], H.nphi,
                    H.ntheta, H.ss_factor, H.beam_spec.c_str(), nE);
        for (size_t b = 0; b < beams.size(); b++)
            std::printf("beam %zu: gantry %.6f couch %.6f coll %.6f rad, iso %g %g %g, sad %g, fluence %dx%d (%s)\n", b,
                        beams[b].b.azimuth, beams[b].b.zenith, beams[b].b.coll, beams[b].b.isocenter[0],
                        beams[b].b.isocenter[1], beams[b].b.isocenter[2], beams[b].b.sad, beams[b].b.fmap_size[0],
                        beams[b].b.fmap_size[1], beams[b].fmap_fname.c_str());
    }
    if (O.dry_run) {
        std::printf("dry run: inputs read in %.1f ms; cone angles from %s\n", t_read - t0,
                    angle_files ? "the temp directory" : "the kernel build");
        return 0;
    }
    if (O.ndevices > 1 && O.verbose) std::printf("--ndevices=%d: every beam runs on device %d\n", O.ndevices, O.device);

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
    std::vector<float> dose(nvox, 0.f);
    double t_set = 0, t_dose = 0;
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
        // max_rev_size 0: derived as initCudaConstandTex does (host.cu:248-258),
        // which overwrites the header's value there too
        ee_conv_params cp = {H.ntheta, H.nphi, H.nradii, H.latspacing, H.longspacing, H.penumbra, {0, 0, 0}};
        if ((rc = check(ee_set_kernel_table(ctx, &cp, radii, cum.data(), theta.data(), phi.data()),
                        "setting the kernel table")))
            break;
        if (O.kernel == "exp") {
            std::vector<float> params((size_t)H.ntheta * 4);
            if ((rc = check(ee_fit_exp_kernel(H.ntheta, EE_DSA_NRADII, radii, cum.data(), params.data(), nullptr),
                            "fitting the kernel")))
                break;
            if ((rc = check(ee_set_kernel_exp(ctx, params.data()), "setting the exp kernel"))) break;
        }
        if ((rc = check(ee_set_terma_supersampling(ctx, H.ss_factor > 0 ? (int)H.ss_factor : 1),
                        "setting TERMA supersampling")))
            break;
        t_set = now_ms();
        std::vector<ee_beam> eb;
        std::vector<float> fl;
        for (const Beam& B : beams) {
            eb.push_back(B.b);
            fl.insert(fl.end(), B.fluence.begin(), B.fluence.end());
        }
        if ((rc = check(ee_beam_dose(ctx, eb.data(), (int)eb.size(), fl.data(), dose.data(), EE_DOSE_SUM),
                        "computing the dose")))
            break;
        t_dose = now_ms();
    } while (false);
    ee_destroy(ctx);
    if (rc) return rc;

    // ---- output: <dir>/<stem>.raw
    std::string dir = ".", stem = O.out;
    const size_t slash = O.out.find_last_of('/');
    if (slash != std::string::npos) {
        dir = O.out.substr(0, slash);
        stem = O.out.substr(slash + 1);
    }
    const size_t dot = stem.find_last_of('.');
    if (dot != std::string::npos && dot > 0) stem = stem.substr(0, dot);
    if (mkdirs(dir)) return fail("cannot create the output directory", dir);
    const std::string raw = dir + "/" + stem + ".raw";
    FILE* f = std::fopen(raw.c_str(), "wb");
    if (!f) return fail("cannot open the output file", raw);
    const size_t put = std::fwrite(dose.data(), sizeof(float), nvox, f);
    std::fclose(f);
    if (put != nvox) return fail("short write", raw);
    std::printf("Data written to \"%s\" (%zu beams, %s kernel); Dose.h5 not written (no HDF5 library)\n", raw.c_str(),
                beams.size(), O.kernel.c_str());
    if (O.timing)
        std::printf("timing [ms]: read inputs %.1f, kernel + set-up %.1f, dose %.1f, total %.1f\n", t_read - t0,
                    t_set - t_read, t_dose - t_set, now_ms() - t0);
    return 0;
}
