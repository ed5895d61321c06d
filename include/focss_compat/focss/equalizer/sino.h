/* Reference header name focss/equalizer/sino.h mapped onto the GPU facade, so callers of
 * the reference API build against libfocss_gpu with only an include-path
 * change (-I include/focss_compat). */
#ifndef FOCSS_COMPAT_EQUALIZER_SINO_H_
#define FOCSS_COMPAT_EQUALIZER_SINO_H_
#include "../../../focss_gpu.hpp"
#endif
