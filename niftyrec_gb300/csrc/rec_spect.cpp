// rec_spect: MLEM / OSEM reconstruction of a SPECT sinogram from the command
// line, with the options of the reference's apps/command_line_tools/rec_spect.cpp:
// NIfTI sinogram [N x M x n_cameras] in, NIfTI activity [N x M x N] out, the
// library's PSF helpers (et_array_calculate_size_psf / et_array_make_psf),
// et_array_mlem for subsets <= 1 and et_array_osem otherwise.  Unlike the
// reference, which parses --attenuation but never loads it
// (rec_spect.cpp:535-549), a given attenuation map is read and used.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "et_array_interface.h"

namespace {

const char* kVersion = "niftyrec-gb300 rec_spect 1.0";

struct Option {
  char short_flag;
  const char* long_flag;
  const char* help;
  bool is_switch;
  std::string value;
};

// Defaults of the reference's TCLAP declarations (rec_spect.cpp:379-396).
std::vector<Option> options() {
  return {
      {'s', "sinogram", "Sinogram data file to reconstruct [N x M x n_cameras] (.nii, .nii.gz); required", false, ""},
      {'o', "output", "Output file name of the reconstructed image [N x M x N] (.nii, .nii.gz); required", false, ""},
      {'a', "attenuation", "Attenuation map image [N x M x N]", false, "none"},
      {'c', "firstcamera", "Position of the first camera in degrees (0.0)", false, "0.0"},
      {'C', "lastcamera", "Position of the last camera in degrees (180.0)", false, "180.0"},
      {'x', "axis", "Axis of rotation of the gamma camera [0, 1, 2] (0)", false, "0"},
      {'f', "fwhm0", "FWHM of the PSF at distance dist0 in pixels (3.0)", false, "3.0"},
      {'F', "fwhm1", "FWHM of the PSF at distance dist1 in pixels (3.0)", false, "3.0"},
      {'e', "efficiency0", "Efficiency of the collimator / detector response at dist0 (0.9)", false, "0.9"},
      {'E', "efficiency1", "Efficiency of the collimator / detector response at dist1 (0.9)", false, "0.9"},
      {'d', "dist0", "Distance of PSF characterisation 0 in pixels (10.0)", false, "10.0"},
      {'D', "dist1", "Distance of PSF characterisation 1 in pixels (10.0)", false, "10.0"},
      {'r', "radius", "Radius of rotation of the gamma camera in pixels (20.0)", false, "20.0"},
      {'i', "iterations", "MLEM / OSEM iterations (20)", false, "20"},
      {'u', "subsets", "Number of OSEM subsets; 0 or 1 for MLEM (16)", false, "16"},
      {'g', "gpu_off", "GPU acceleration off (accepted; the library always uses the GPU)", true, "0"},
      {'v', "verbose", "Print verbose information", true, "0"},
  };
}

void usage(const std::vector<Option>& opts) {
  std::printf("%s\nMaximum likelihood expectation maximisation (MLEM) and ordered subsets (OSEM) reconstruction "
              "of SPECT sinogram data.\n\nUSAGE: rec_spect -s <sinogram> -o <output> [options]\n\n", kVersion);
  for (const Option& o : opts)
    std::printf("  -%c, --%-12s %s%s\n", o.short_flag, o.long_flag, o.is_switch ? "" : "<value>  ", o.help);
  std::printf("  --xml            Print the parameter description as XML\n  -h, --help       This text\n");
}

void print_xml(const std::vector<Option>& opts) {
  std::printf("<?xml version=\"1.0\" encoding=\"utf-8\"?>\n<executable>\n  <title>rec_spect</title>\n"
              "  <description>MLEM / OSEM reconstruction of SPECT sinogram data</description>\n"
              "  <parameters>\n");
  for (const Option& o : opts)
    std::printf("    <%s><name>%s</name><flag>%c</flag><longflag>%s</longflag><description>%s</description>"
                "<default>%s</default></%s>\n",
                o.is_switch ? "boolean" : "string", o.long_flag, o.short_flag, o.long_flag, o.help,
                o.value.c_str(), o.is_switch ? "boolean" : "string");
  std::printf("  </parameters>\n</executable>\n");
}

bool has_suffix(const std::string& s, const char* suffix) {
  const size_t n = std::strlen(suffix);
  return s.size() >= n && s.compare(s.size() - n, n, suffix) == 0;
}

bool is_nifti(const std::string& s) { return has_suffix(s, ".nii") || has_suffix(s, ".nii.gz"); }

}  // namespace

int main(int argc, char** argv) {
  std::vector<Option> opts = options();
  if (argc == 2 && std::strcmp(argv[1], "--xml") == 0) {
    print_xml(opts);
    return 0;
  }
  std::map<std::string, std::string> seen;
  for (int i = 1; i < argc; ++i) {
    std::string arg = argv[i];
    if (arg == "-h" || arg == "--help") {
      usage(opts);
      return 0;
    }
    if (arg == "--version") {
      std::printf("%s\n", kVersion);
      return 0;
    }
    Option* hit = nullptr;
    std::string inline_value;
    bool has_inline = false;
    for (Option& o : opts) {
      const std::string lf = std::string("--") + o.long_flag;
      if (arg == lf || (arg.size() == 2 && arg[0] == '-' && arg[1] == o.short_flag)) {
        hit = &o;
      } else if (arg.compare(0, lf.size() + 1, lf + "=") == 0) {
        hit = &o;
        inline_value = arg.substr(lf.size() + 1);
        has_inline = true;
      }
      if (hit) break;
    }
    if (!hit) {
      std::fprintf(stderr, "error: unknown argument %s\n", arg.c_str());
      usage(opts);
      return 1;
    }
    if (hit->is_switch) {
      hit->value = "1";
    } else if (has_inline) {
      hit->value = inline_value;
    } else if (i + 1 < argc) {
      hit->value = argv[++i];
    } else {
      std::fprintf(stderr, "error: missing value for --%s\n", hit->long_flag);
      return 1;
    }
    seen[hit->long_flag] = hit->value;
  }
  auto get = [&](const char* name) -> std::string {
    for (const Option& o : opts)
      if (std::strcmp(o.long_flag, name) == 0) return o.value;
    return "";
  };
  const std::string sino_name = get("sinogram"), out_name = get("output"), att_name = get("attenuation");
  if (!seen.count("sinogram") || !seen.count("output")) {
    std::fprintf(stderr, "error: --sinogram and --output are required\n");
    usage(opts);
    return 1;
  }
  const float first = std::strtof(get("firstcamera").c_str(), nullptr);
  const float last = std::strtof(get("lastcamera").c_str(), nullptr);
  const unsigned axis = static_cast<unsigned>(std::atoi(get("axis").c_str()));
  const float fwhm0 = std::strtof(get("fwhm0").c_str(), nullptr), fwhm1 = std::strtof(get("fwhm1").c_str(), nullptr);
  const float eff0 = std::strtof(get("efficiency0").c_str(), nullptr);
  const float eff1 = std::strtof(get("efficiency1").c_str(), nullptr);
  const float dist0 = std::strtof(get("dist0").c_str(), nullptr), dist1 = std::strtof(get("dist1").c_str(), nullptr);
  const float radius = std::strtof(get("radius").c_str(), nullptr);
  const int iterations = std::atoi(get("iterations").c_str());
  const int subsets = std::atoi(get("subsets").c_str());
  const int gpu = get("gpu_off") == "1" ? 0 : 1;

  if (!is_nifti(sino_name)) {
    std::printf(has_suffix(sino_name, ".nrrd") ? "NRRD file format not supported.\n" : "Unknown file format\n");
    return 1;
  }
  if (!is_nifti(out_name)) {
    std::printf(has_suffix(out_name, ".nrrd") ? "NRRD file format not supported.\n" : "Unknown file format\n");
    return 1;
  }
  std::printf("Nifti sinogram file: %s\n", sino_name.c_str());
  int dims[8];
  if (nrgb_nifti_info(sino_name.c_str(), dims) != 0 || dims[0] < 2) {
    std::printf("Couldn't load the sinogram %s\n", sino_name.c_str());
    return 1;
  }
  const unsigned size_x = dims[1], size_y = dims[2];
  const int n_cameras = dims[0] >= 3 ? dims[3] : 1;
  std::vector<float> sino(static_cast<size_t>(size_x) * size_y * n_cameras);
  if (nrgb_nifti_read(sino_name.c_str(), sino.data(), static_cast<long long>(sino.size())) != 0) {
    std::printf("Couldn't load the sinogram %s\n", sino_name.c_str());
    return 1;
  }
  const size_t nvox = static_cast<size_t>(size_x) * size_y * size_x;
  std::vector<float> attenuation;
  int use_attenuation = 0;
  if (att_name != "none") {
    int adims[8];
    if (!is_nifti(att_name) || nrgb_nifti_info(att_name.c_str(), adims) != 0 || adims[1] != static_cast<int>(size_x) ||
        adims[2] != static_cast<int>(size_y) || adims[3] != static_cast<int>(size_x)) {
      std::printf("Couldn't load the attenuation map %s (expected [%u x %u x %u])\n", att_name.c_str(), size_x,
                  size_y, size_x);
      return 1;
    }
    attenuation.resize(nvox);
    if (nrgb_nifti_read(att_name.c_str(), attenuation.data(), static_cast<long long>(nvox)) != 0) {
      std::printf("Couldn't load the attenuation map %s\n", att_name.c_str());
      return 1;
    }
    use_attenuation = 1;
  }
  std::printf("=============== NiftyRec SPECT Parameters ===============\n");
  std::printf("Sinogram file name:       %s\n", sino_name.c_str());
  std::printf("Output file name:         %s\n", out_name.c_str());
  std::printf("Attenuation file name:    %s\n", att_name.c_str());
  std::printf("First camera:             %g\n", first);
  std::printf("Last camera:              %g\n", last);
  std::printf("Rotation axis:            %u\n", axis);
  std::printf("PSF distance 0 [pixels]:  %g\n", dist0);
  std::printf("PSF FWHM 0 [pixels]:      %g\n", fwhm0);
  std::printf("PSF efficiency 0:         %g\n", eff0);
  std::printf("PSF distance 1 [pixels]:  %g\n", dist1);
  std::printf("PSF FWHM 1 [pixels]:      %g\n", fwhm1);
  std::printf("PSF efficiency 1:         %g\n", eff1);
  std::printf("Rotation radius [pixels]: %g\n", radius);
  std::printf("Sinogram size X [pixels]: %u\n", size_x);
  std::printf("Sinogram size Y [pixels]: %u\n", size_y);
  std::printf("Number of projections:    %d\n", n_cameras);
  std::printf("Subsets:                  %d\n", subsets);
  std::printf("Iterations:               %d\n", iterations);
  std::printf("Use GPU:                  %d\n", gpu);
  std::printf("=========================================================\n");

  unsigned psf_x = 0, psf_y = 0;
  if (et_array_calculate_size_psf(&psf_x, &psf_y, fwhm0, eff0, dist0, fwhm1, eff1, dist1) != 0) {
    std::fprintf(stderr, "rec_spect: Error creating PSF.\n");
    return 1;
  }
  std::vector<float> psf(static_cast<size_t>(psf_x) * psf_y * size_x);
  if (et_array_make_psf(psf.data(), psf_x, psf_y, fwhm0, eff0, dist0, fwhm1, eff1, dist1, size_x) != 0) {
    std::fprintf(stderr, "rec_spect: Error creating PSF.\n");
    return 1;
  }
  std::vector<float> activity(nvox);
  const float bg = 0.0f, bg_att = 0.0f, eps = 0.0000001f;  // rec_spect.cpp:27-29
  float* att = use_attenuation ? attenuation.data() : nullptr;
  const int status =
      subsets <= 1
          ? et_array_mlem(activity.data(), size_x, size_y, sino.data(), n_cameras, first, last, axis, iterations,
                          use_attenuation, att, 1, psf.data(), psf_x, psf_y, bg, bg_att, eps, gpu)
          : et_array_osem(activity.data(), size_x, size_y, static_cast<unsigned>(subsets), sino.data(), n_cameras,
                          first, last, axis, iterations, use_attenuation, att, 1, psf.data(), psf_x, psf_y, bg, bg_att,
                          eps, gpu);
  if (status != 0) {
    std::fprintf(stderr, "rec_spect: reconstruction failed.\n ");
    return 1;
  }
  std::printf("Nifti output file: %s\n", out_name.c_str());
  const int odims[4] = {3, static_cast<int>(size_x), static_cast<int>(size_y), static_cast<int>(size_x)};
  if (nrgb_nifti_write(out_name.c_str(), activity.data(), odims) != 0) {
    std::printf("Couldn't write %s\n", out_name.c_str());
    return 1;
  }
  return 0;
}
