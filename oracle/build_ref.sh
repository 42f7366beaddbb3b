#!/bin/sh
# Compiles the reference's own cubic kernel and quaternion-Jacobian sources (they need only
# Eigen, which the reference vendors) together with oracle/ref_pin.cpp, and its regular
# triangle surface sampler with oracle/ref_sampling.cpp, into oracle/_ref/.
# The DiffDFSPH step itself needs stand-ins for the three libraries the reference fetches at
# configure time (CompactNSearch, GenericParameters, Discregrid): oracle/build_ref_step.sh.
set -e
# The checkout comes from the first argument, else DIFFFR_REFERENCE, else ../reference
# beside the repository.
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${1:-${DIFFFR_REFERENCE:-$HERE/../../reference}}
OUT=$(cd "$(dirname "$0")" && pwd)/_ref
mkdir -p "$OUT"
SRC=$(cd "$(dirname "$0")" && pwd)/ref_pin.cpp
INC="-I$REF -I$REF/SPlisHSPlasH -I$REF/extern/eigen"
for prec in double float; do
  DEF=""
  [ "$prec" = double ] && DEF="-DUSE_DOUBLE"
  g++ -O2 -std=c++17 -ffp-contract=off $DEF $INC "$SRC" "$REF/SPlisHSPlasH/SPHKernels.cpp" \
      "$REF/SPlisHSPlasH/GradientUtils.cpp" -o "$OUT/ref_pin_$prec"
done
# the regular triangle surface sampler (needs only Common.h and Eigen), double build
g++ -O2 -std=c++17 -ffp-contract=off -DUSE_DOUBLE $INC "$(dirname "$SRC")/ref_sampling.cpp" \
    "$REF/SPlisHSPlasH/Utilities/RegularTriangleSampling.cpp" -o "$OUT/ref_sampling_double"
echo "$OUT"
