// Drives the UNMODIFIED reference library's path segment storage
// (oracle/_ref/libopenpgl_ref.so) through its public C++ wrapper, path by
// path, the way a renderer does, to produce golden samples and pixel
// estimates (tests/golden/paths.npz).  Test infrastructure; never shipped.
//
// usage: ref_paths <paths.bin> <out_prefix> <maxDistance>
// paths.bin : u64 numPaths, u64 begin[numPaths + 1], then the segments
//             (PGLPathSegmentData, 136 bytes each)
// outputs   : <out_prefix>.counts.bin  u32 [8][numPaths] samples per path for
//                                      flag set f (bit 0 useNEEMiWeights,
//                                      bit 1 guideDirectLight, bit 2
//                                      rrAffectsDirectContribution)
//             <out_prefix>.samples.bin the samples, flag set by flag set, path by path
//             <out_prefix>.pixel.bin   f32 [2][numPaths][3] CalculatePixelEstimate
//                                      (rrAffectsDirectContribution false, true)
#include <openpgl/cpp/OpenPGL.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

int main(int argc, char **argv) {
  if (argc < 4) {
    std::fprintf(stderr, "usage: %s paths.bin out_prefix maxDistance\n", argv[0]);
    return 2;
  }
  FILE *f = std::fopen(argv[1], "rb");
  if (!f) return 1;
  uint64_t numPaths = 0;
  if (std::fread(&numPaths, 8, 1, f) != 1) return 1;
  std::vector<uint64_t> begin(numPaths + 1);
  if (std::fread(begin.data(), 8, begin.size(), f) != begin.size()) return 1;
  std::vector<PGLPathSegmentData> segs(begin[numPaths]);
  if (std::fread(segs.data(), sizeof(PGLPathSegmentData), segs.size(), f) != segs.size()) return 1;
  std::fclose(f);
  const std::string prefix = argv[2];
  const float maxDistance = float(std::atof(argv[3]));

  openpgl::cpp::PathSegmentStorage storage;
  size_t longest = 1;
  for (uint64_t p = 0; p < numPaths; ++p) longest = std::max<size_t>(longest, begin[p + 1] - begin[p]);
  storage.Reserve(longest + 1);
  storage.SetMaxDistance(maxDistance);
  std::vector<uint32_t> counts(8 * numPaths);
  std::vector<PGLSampleData> samples;
  std::vector<float> pixel(2 * numPaths * 3);
  for (int fl = 0; fl < 8; ++fl) {
    for (uint64_t p = 0; p < numPaths; ++p) {
      storage.Clear();
      for (uint64_t s = begin[p]; s < begin[p + 1]; ++s) {
        PGLPathSegmentData *seg = storage.NextSegment();
        *seg = segs[s];
      }
      storage.PrepareSamples((fl & 1) != 0, (fl & 2) != 0, (fl & 4) != 0);
      size_t n = 0;
      const PGLSampleData *out = storage.GetSamples(n);
      counts[fl * numPaths + p] = uint32_t(n);
      samples.insert(samples.end(), out, out + n);
      if (fl < 2) {
        const pgl_vec3f c = storage.CalculatePixelEstimate(fl == 1);
        float *o = &pixel[(fl * numPaths + p) * 3];
        o[0] = c.x;
        o[1] = c.y;
        o[2] = c.z;
      }
    }
  }
  FILE *fc = std::fopen((prefix + ".counts.bin").c_str(), "wb");
  std::fwrite(counts.data(), 4, counts.size(), fc);
  std::fclose(fc);
  FILE *fs = std::fopen((prefix + ".samples.bin").c_str(), "wb");
  std::fwrite(samples.data(), sizeof(PGLSampleData), samples.size(), fs);
  std::fclose(fs);
  FILE *fp = std::fopen((prefix + ".pixel.bin").c_str(), "wb");
  std::fwrite(pixel.data(), 4, pixel.size(), fp);
  std::fclose(fp);
  return 0;
}
