// hdog_stage_test.cpp -- drop-in for the reference's stage programs test/Normalize_test,
// DoG_test, Hessian_test, CCL_test and Regional_test (test/*_test.cpp), which
// script/HDoG_intermediate.py:25-104 runs to dump a substack's intermediate volumes.
//
//   Normalize_test PARAM [EROSION DILATION NORMALIZED]   (or [NORMALIZED])
//   DoG_test       PARAM [DOG]  (or [NORMALIZED DOG])
//   Hessian_test   PARAM [DOG PD [HESSIAN]]
//   CCL_test       PARAM        -> labels.bin, hessian_pd.bin
//   Regional_test  PARAM        -> labels.bin, normalized.bin and the per-region files
//
// The program is chosen by the name it is run under (the build links the five names to
// this binary) or by a first argument naming it (`hdog_stage_test DoG_test PARAM ...`).
// The parameter file must hold one stack of exactly `depth` slices (exit 2 otherwise), the
// files written, their names, element types and the argument-count and `verbose` rules are
// the reference programs' (including that Hessian_test with verbose set and fewer than
// three output names writes nothing, and that CCL_test runs on device 0).  Every volume is
// raw, depth x height x width, x fastest.
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/hdog.h"
#include "json_min.hpp"

namespace json = hdog::json;

namespace {

int die(int code, const std::string &msg) {
  std::printf("%s\n", msg.c_str());
  return code;
}

// saveImage (src/3D/utils.h:176-185): raw elements, exit 2 when the file cannot be opened.
bool save(const void *data, size_t elem, size_t n, const std::string &path) {
  FILE *f = std::fopen(path.c_str(), "wb");
  if (!f) {
    std::printf("Unable to open %s\n", path.c_str());
    return false;
  }
  std::fwrite(data, elem, n, f);
  std::fclose(f);
  return true;
}

struct Dev {   // device buffer owned by the program
  void *p = nullptr;
  explicit Dev(size_t bytes) { hdog_device_alloc(&p, bytes); }
  ~Dev() { if (p) hdog_device_free(p); }
  template <class T> T *as() const { return static_cast<T *>(p); }
};

template <class T>
bool fetch_save(const void *dptr, size_t n, const std::string &path) {
  std::vector<T> h(n);
  if (n && hdog_memcpy(h.data(), dptr, n * sizeof(T), nullptr) != HDOG_OK) return false;
  hdog_stream_sync(nullptr);
  return save(h.data(), sizeof(T), n, path);
}

}  // namespace

int main(int argc, char **argv) {
  std::string prog = argv[0];
  const size_t slash = prog.find_last_of('/');
  if (slash != std::string::npos) prog = prog.substr(slash + 1);
  const char *names[] = {"Normalize_test", "DoG_test", "Hessian_test", "CCL_test", "Regional_test"};
  bool named = false;
  for (const char *n : names) named |= prog == n;
  if (!named && argc >= 2) {   // hdog_stage_test NAME PARAM ...
    prog = argv[1];
    argv++;
    argc--;
  }
  int which = -1;
  for (int i = 0; i < 5; i++)
    if (prog == names[i]) which = i;
  if (which < 0 || argc < 2)
    return die(2, "Usage: {Normalize,DoG,Hessian,CCL,Regional}_test PARAM_FILE [outputs...]\n"
                  "   or: hdog_stage_test NAME_test PARAM_FILE [outputs...]");

  hdog_params p;
  if (hdog_params_load_json(argv[1], &p) != HDOG_OK) return die(2, hdog_last_error());
  // the stack list and `verbose`, read as loadParamFile does (src/3D/utils.h:95-157)
  std::ifstream in(argv[1], std::ios::binary);
  std::stringstream ss;
  ss << in.rdbuf();
  json::Value root;
  std::string err;
  if (!json::Parser(ss.str()).parse(root, err)) return die(2, "parameter file: " + err);
  const json::Value *v = root.get("verbose");
  const bool verbose = v && ((v->kind == json::Value::Bool && v->b) || (v->kind == json::Value::Number && v->num != 0));
  const json::Value *st = root.get("stacks");
  if (!st || st->kind != json::Value::Array || st->arr.size() != 1)
    return die(2, "A single stack should be provided!");
  const json::Value *srcs = st->arr[0].get("src_paths");
  const int length = srcs && srcs->kind == json::Value::Array ? (int)srcs->arr.size() : 0;
  if (length != p.depth) return die(2, "depth(=" + std::to_string(length) + ") should be " + std::to_string(p.depth));
  if (which == 3) p.dev_id = 0;        // CCL_test initializes device 0 whatever devID says
  if (which == 4) p.is_ave_mode = 0;   // Regional_test reduces with MaxNormalized

  std::printf("sigma_xy1: %g\tsigma_z1: %g\tsigma_xy2: %g\tsigma_z2: %g\n", p.sigma_xy_small, p.sigma_z_small,
              p.sigma_xy_large, p.sigma_z_large);
  std::printf("radius_large_xy: %d\tradius_large_z: %d\n", p.radius_norm_xy, p.radius_norm_z);

  // loadImage (src/3D/utils.h:160-173): the first W*H values of each slice file
  const size_t plane = (size_t)p.width * p.height, n = plane * p.depth;
  std::vector<uint16_t> img(n, 0);
  for (int z = 0; z < p.depth; z++) {
    const std::string path = srcs->arr[z].str;
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) return die(2, "Unable to open " + path);
    const size_t got = std::fread(img.data() + z * plane, sizeof(uint16_t), plane, f);
    (void)got;   // a short file leaves the rest of its slice zero
    std::fclose(f);
  }

  hdog_ctx *ctx = nullptr;
  if (hdog_ctx_create(&p, 1, &ctx) != HDOG_OK) return die(1, hdog_last_error());
  int rc = 0;
  {
    Dev d_img(n * 2), d_norm(n * 4), d_ero(n * 4), d_dil(n * 4), d_dog(n * 4), d_pd(n), d_hess(n * 4 * 6),
        d_lab(n * 4);
    auto ok = [&](int r) {
      if (r != HDOG_OK) {
        std::fprintf(stderr, "%s\n", hdog_last_error());
        rc = 1;
      }
      return r == HDOG_OK;
    };
    if (!ok(hdog_memcpy(d_img.p, img.data(), n * 2, nullptr))) goto done;
    if (!ok(hdog_normalize_parts(ctx, d_img.as<uint16_t>(), d_norm.as<float>(), d_ero.as<float>(),
                                 d_dil.as<float>(), nullptr)))
      goto done;
    if (which == 0) {   // test/Normalize_test.cpp:104-121
      bool w = true;
      if (verbose) {
        if (argc == 5) {
          w = fetch_save<float>(d_ero.p, n, argv[2]) && fetch_save<float>(d_dil.p, n, argv[3]) &&
              fetch_save<float>(d_norm.p, n, argv[4]);
        } else if (argc == 3) {
          w = fetch_save<float>(d_ero.p, n, "./erosion_l.bin") && fetch_save<float>(d_dil.p, n, "./dilation_l.bin") &&
              fetch_save<float>(d_norm.p, n, argv[2]);
        } else {
          w = fetch_save<float>(d_ero.p, n, "./erosion_l.bin") && fetch_save<float>(d_dil.p, n, "./dilation_l.bin") &&
              fetch_save<float>(d_norm.p, n, "./normalized.bin");
        }
      } else {
        w = fetch_save<float>(d_norm.p, n, argc == 3 ? argv[2] : "./normalized.bin");
      }
      if (!w) rc = 2;
      goto done;
    }
    if (!ok(hdog_dog(ctx, d_norm.as<float>(), d_dog.as<float>(), nullptr))) goto done;
    if (which == 1) {   // test/DoG_test.cpp:125-135
      bool w = true;
      if (argc == 3) {
        w = fetch_save<float>(d_dog.p, n, argv[2]);
      } else if (argc == 4) {
        w = fetch_save<float>(d_norm.p, n, argv[2]) && fetch_save<float>(d_dog.p, n, argv[3]);
      } else {
        w = fetch_save<float>(d_dog.p, n, "./dog.bin");
        if (verbose) w = w && fetch_save<float>(d_norm.p, n, "./normalized.bin");
      }
      if (!w) rc = 2;
      goto done;
    }
    if (!ok(hdog_hessian_pd(ctx, d_dog.as<float>(), d_pd.as<uint8_t>(), verbose ? d_hess.as<float>() : nullptr,
                            nullptr)))
      goto done;
    if (which == 2) {   // test/Hessian_test.cpp:139-157
      bool w = true;
      if (verbose) {
        if (argc == 5) {
          w = fetch_save<float>(d_dog.p, n, argv[2]) && fetch_save<uint8_t>(d_pd.p, n, argv[3]) &&
              fetch_save<float>(d_hess.p, n * 6, argv[4]);
        } else if (argc == 4) {
          w = fetch_save<float>(d_dog.p, n, argv[2]) && fetch_save<uint8_t>(d_pd.p, n, argv[3]) &&
              fetch_save<float>(d_hess.p, n * 6, "hessian.bin");
        }
      } else {
        if (argc == 4) {
          w = fetch_save<float>(d_dog.p, n, argv[2]) && fetch_save<uint8_t>(d_pd.p, n, argv[3]);
        } else {
          w = fetch_save<float>(d_dog.p, n, "dog.bin") && fetch_save<uint8_t>(d_pd.p, n, "hessian_pd.bin");
        }
      }
      if (!w) rc = 2;
      goto done;
    }
    if (!ok(hdog_ccl(ctx, d_pd.as<uint8_t>(), d_lab.as<int32_t>(), nullptr))) goto done;
    if (which == 3) {   // test/CCL_test.cpp:137-139
      if (!(fetch_save<int32_t>(d_lab.p, n, "labels.bin") && fetch_save<uint8_t>(d_pd.p, n, "hessian_pd.bin"))) rc = 2;
      goto done;
    }
    // Regional_test (test/Regional_test.cpp:180-235): region 0 (background) is not written
    hdog_regions R;
    if (!ok(hdog_regional_features(ctx, d_lab.as<int32_t>(), d_norm.as<float>(), d_dog.as<float>(), &R, nullptr)))
      goto done;
    std::printf("num_regions: %lld\n", (long long)R.num_regions);
    std::printf("Saving...\n");
    const size_t nr = R.num_regions > 0 ? (size_t)R.num_regions - 1 : 0;
    std::vector<uint32_t> cnt(nr);
    std::vector<uint16_t> size16(nr);
    if (nr) hdog_memcpy(cnt.data(), R.count + 1, nr * 4, nullptr);
    hdog_stream_sync(nullptr);
    for (size_t i = 0; i < nr; i++) size16[i] = (uint16_t)(cnt[i] & 0xFFFFu);
    bool w = fetch_save<int32_t>(d_lab.p, n, "labels.bin") && fetch_save<float>(d_norm.p, n, "normalized.bin") &&
             fetch_save<int32_t>(R.label + 1, nr, "labels_region.bin") &&
             save(size16.data(), 2, nr, "size_region.bin") &&
             fetch_save<float>(R.intensity + 1, nr, "max_normalized_region.bin") &&
             fetch_save<float>(R.eigen + 1, nr, "structureness_region.bin") &&
             fetch_save<float>(R.eigen + R.pitch + 1, nr, "blobness_region.bin") &&
             fetch_save<float>(R.centroid + 1, nr, "centroid_x.bin") &&
             fetch_save<float>(R.centroid + R.pitch + 1, nr, "centroid_y.bin") &&
             fetch_save<float>(R.centroid + 2 * R.pitch + 1, nr, "centroid_z.bin");
    if (!w) rc = 2;
  }
done:
  hdog_ctx_destroy(ctx);
  return rc;
}
