#!/bin/sh
# Compiles the reference's own cubic kernel and quaternion-Jacobian sources (they need only
# Eigen, which the reference vendors) together with oracle/ref_pin.cpp into oracle/_ref/.
# The rest of the reference is not buildable here: its hot-path translation units include
# CompactNSearch, GenericParameters and Discregrid, which its CMake fetches by git.
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
echo "$OUT"
