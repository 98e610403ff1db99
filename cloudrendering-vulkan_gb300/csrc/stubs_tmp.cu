#include "vcr_internal.h"
namespace vcr {
void nrc_free(vcr_ctx*) {}
}
