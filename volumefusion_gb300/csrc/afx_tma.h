// afx_tma.h -- tensor-map encoding (driver entry point looked up once) for the TMA tile loads.
#pragma once

#include <cuda.h>

namespace afx {

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// cuTensorMapEncodeTiled, or nullptr when the driver does not provide it.
EncodeTiledFn encode_fn();

}  // namespace afx
