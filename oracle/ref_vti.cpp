// C entry point over the reference's own VTI reader (src/sdf_reader.cpp, compiled unmodified from
// the reference checkout by oracle/build_ref.sh). Test infrastructure only: pins pnm_read_vti.
#include <cstdlib>
#include <cstring>
#include <exception>

#include "sdf_reader.h"

extern "C" {

// Returns 0 and a malloc'd copy of the values (x fastest), or 1 when read_vti throws.
int ref_read_vti(const char* path, int* dims_xyz, float* origin_xyz, float* spacing_xyz,
                 float** values, long long* n) {
  try {
    SDFData d = SDFReader::read_vti(path);
    for (int a = 0; a < 3; ++a) {
      dims_xyz[a] = d.resolution[a];
      origin_xyz[a] = d.origin[a];
      spacing_xyz[a] = d.spacing[a];
    }
    *n = (long long)d.sdf_values.size();
    *values = (float*)std::malloc(d.sdf_values.size() * sizeof(float) + 4);
    std::memcpy(*values, d.sdf_values.data(), d.sdf_values.size() * sizeof(float));
    return 0;
  } catch (const std::exception&) {
    return 1;
  }
}

void ref_vti_free(void* p) { std::free(p); }

}  // extern "C"
