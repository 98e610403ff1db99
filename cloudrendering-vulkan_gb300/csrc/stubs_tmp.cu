#include "vcr_internal.h"
namespace vcr {
void ppm_free(vcr_ctx*) {}
void nrc_free(vcr_ctx*) {}
}
