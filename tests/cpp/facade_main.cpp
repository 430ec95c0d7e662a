// Test harness around the C++ binding shown in INTEGRATION.md section 2: the test
// concatenates that block and this file into one translation unit.
//   facade_main <points.f32> <sx> <bsx> <numIter> <dt> <out.bin>
// out.bin: int64 nActive, int32 activeBlocks[nActive], float32 density[nActive*bsx^3],
// double dots[3]; the status of surfaceOnGb300 is the exit code.
#include <stdio.h>
#include <stdlib.h>

int main(int argc, char **argv) {
  if (argc != 7) return 2;
  FILE *f = fopen(argv[1], "rb");
  if (!f) return 3;
  fseek(f, 0, SEEK_END);
  const long bytes = ftell(f);
  fseek(f, 0, SEEK_SET);
  std::vector<float> pts((size_t)bytes / 4);
  if (fread(pts.data(), 4, pts.size(), f) != pts.size()) return 3;
  fclose(f);
  const int s = atoi(argv[2]), bsx = atoi(argv[3]), numIter = atoi(argv[4]);
  const float dt = (float)atof(argv[5]);
  std::vector<int> active;
  std::vector<float> density;
  double dots[3] = {0, 0, 0};
  const int rc = surfaceOnGb300(pts.data(), (int64_t)(pts.size() / 3), s, s, s, bsx, numIter, dt, active, density,
                                dots);
  if (rc) return rc < 0 ? -rc : rc;
  FILE *o = fopen(argv[6], "wb");
  if (!o) return 4;
  const int64_t na = (int64_t)active.size();
  fwrite(&na, 8, 1, o);
  fwrite(active.data(), 4, active.size(), o);
  fwrite(density.data(), 4, density.size(), o);
  fwrite(dots, 8, 3, o);
  fclose(o);
  return 0;
}
