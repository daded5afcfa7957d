#!/bin/sh
# Compiles the RBMonGPU reference's own sources (read in place, never copied) and
# links them with ref_harness.cu into oracle/_ref/ref_harness.  Only the host path
# (objects built with gpu=false) is exercised; the device code is compiled because
# the reference's translation units contain it.  Outputs go to oracle/_ref only.
set -e
HERE=$(cd "$(dirname "$0")/.." && pwd)
# the RBMonGPU checkout: first argument, else $RBMONGPU_REF; nothing to do without one
REF=${1:-$RBMONGPU_REF}
if [ -z "$REF" ] || [ ! -d "$REF/source" ]; then
  echo "build_ref.sh: no RBMonGPU sources given (argument or RBMONGPU_REF); reference harness not built"
  exit 0
fi
OUT="$HERE/_ref"
NVCC=${NVCC:-nvcc}
FLAGS="-std=c++14 -O2 --expt-extended-lambda -gencode arch=compute_100,code=sm_100 \
 -DENABLE_PSI -DENABLE_PSI_DEEP -DENABLE_PSI_PAIR -DENABLE_MONTE_CARLO -DENABLE_EXACT_SUMMATION \
 -I$REF/include -I$HERE/ref/shim -Xcompiler -ffp-contract=off -w"
mkdir -p "$OUT/obj"
UNITS="Array RNGStates quantum_state/Psi quantum_state/PsiDeep quantum_state/PsiPair \
 spin_ensembles/MonteCarloLoop spin_ensembles/ExactSummation operator/Operator \
 network_functions/ExpectationValue network_functions/PsiNorm network_functions/HilbertSpaceDistance \
 network_functions/HilbertSpaceDistance_PsiPair network_functions/PsiVector network_functions/PsiOkVector \
 network_functions/S_matrix network_functions/HilbertSpaceDistance_2nd_order network_functions/DiagDensityOp"
pids=""
for u in $UNITS; do
  o="$OUT/obj/$(echo "$u" | tr / _).o"
  if [ ! -f "$o" ] || [ "$REF/source/$u.cu" -nt "$o" ]; then
    $NVCC $FLAGS -c "$REF/source/$u.cu" -o "$o" &
    pids="$pids $!"
  fi
done
for p in $pids; do wait "$p"; done
$NVCC $FLAGS -D__PYTHONCC__ -c "$HERE/ref/ref_harness.cu" -o "$OUT/obj/ref_harness.o"
$NVCC -o "$OUT/ref_harness" "$OUT"/obj/*.o
echo "built $OUT/ref_harness"
