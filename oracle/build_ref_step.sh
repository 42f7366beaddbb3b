#!/bin/sh
# Builds oracle/_ref/ref_step_{double,float}: the reference's own DiffDFSPH step (its
# sources compiled where they lie in the checkout) driven by oracle/ref_step.cpp, against
# the stand-ins in oracle/refshim/ for the three libraries the reference fetches at
# configure time (GenericParameters, CompactNSearch, Discregrid). Test infrastructure only.
#
# The reference's simulator shell, its other pressure solvers and its other force models are
# not compiled. Functions of those parts that the compiled sources name but this driver
# never reaches stay unresolved: the executable is linked position-dependent with
# unresolved symbols allowed, so such a symbol has address 0 and reaching one would stop the
# program with a fault (the driver never does; its runs are checked for complete output).
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${1:-${DIFFFR_REFERENCE:-$HERE/../../reference}}
OUT=$HERE/_ref
mkdir -p "$OUT"
SP=$REF/SPlisHSPlasH
SRCS="$SP/DiffDFSPH/TimeStepDiffDFSPH.cpp $SP/DiffDFSPH/SimulationDataDiffDFSPH.cpp $SP/TimeStep.cpp
  $SP/Simulation.cpp $SP/FluidModel.cpp $SP/BoundaryModel.cpp $SP/BoundaryModel_Akinci2012.cpp $SP/SPHKernels.cpp
  $SP/GradientUtils.cpp $SP/RigidBodyGradientManager.cpp $SP/TimeManager.cpp $SP/NonPressureForceBase.cpp
  $SP/Viscosity/ViscosityBase.cpp $SP/Viscosity/Viscosity_XSPH.cpp $SP/TriangleMesh.cpp
  $SP/AnimationFieldSystem.cpp $SP/AnimationField.cpp $SP/EmitterSystem.cpp $SP/Emitter.cpp
  $REF/Simulator/SceneConfiguration.cpp $REF/Utilities/ColorfulPrint.cpp"
INC="-I$HERE/refshim -I$REF -I$SP -I$REF/extern/eigen -I$REF/extern"
for prec in double float; do
  DEF="-DEIGEN_DISABLE_UNALIGNED_ARRAY_ASSERT"
  [ "$prec" = double ] && DEF="$DEF -DUSE_DOUBLE"
  OBJ=$OUT/obj_$prec
  mkdir -p "$OBJ"
  objs=""
  for s in $SRCS "$HERE/ref_step.cpp"; do
    o=$OBJ/$(basename "$s" .cpp).o
    g++ -O2 -std=c++17 -fopenmp -ffp-contract=off -fno-pie -w -include cfloat $DEF $INC -c "$s" -o "$o" &
    objs="$objs $o"
  done
  gcc -O2 -fno-pie -w -c "$REF/extern/tinyexpr/tinyexpr.c" -o "$OBJ/tinyexpr.o"
  objs="$objs $OBJ/tinyexpr.o"
  wait
  g++ -no-pie -fopenmp -o "$OUT/ref_step_$prec" $objs -Wl,--unresolved-symbols=ignore-all
done
echo "$OUT"
