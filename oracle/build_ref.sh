#!/bin/sh
# Builds the reference implementation's compiled extension (yaff.pes.ext) from
# the read-only reference checkout into oracle/_ref/.  Test infrastructure only:
# the result is used to generate golden fixtures and to cross-check the oracle
# port; nothing in the product imports it.
#
#   sh oracle/build_ref.sh            (reference at $YAFF_REFERENCE or /root/reference)
#
# The reference's own setup.py is not used (it fails under Cython 3 because of
# implicit relative cimports); cython + gcc are run on its sources directly.
# -ffp-contract=off keeps gcc from fusing multiply-adds on hosts where it would
# (aarch64), so the build reproduces the x86-64 SSE2 arithmetic of the reference.
set -e
REF=${YAFF_REFERENCE:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -f "$REF/yaff/pes/ext.pyx" ]; then
  echo "build_ref: reference sources not found at $REF; nothing built"
  exit 0
fi
PY=${PYTHON:-python3}
SUFFIX=$($PY -c 'import sysconfig;print(sysconfig.get_config_var("EXT_SUFFIX"))')
PYINC=$($PY -c 'import sysconfig;print(sysconfig.get_paths()["include"])')
NPINC=$($PY -c 'import numpy;print(numpy.get_include())')
mkdir -p "$OUT/build" "$OUT/pes"
if [ ! -f "$OUT/pes/ext$SUFFIX" ] || [ "$REF/yaff/pes/ext.pyx" -nt "$OUT/pes/ext$SUFFIX" ]; then
  cython -2 -I "$REF/yaff/pes" "$REF/yaff/pes/ext.pyx" -o "$OUT/build/ext.c"
  P="$REF/yaff/pes"
  gcc -O2 -fPIC -shared -ffp-contract=off -w -I"$PYINC" -I"$NPINC" -I"$P" \
    "$OUT/build/ext.c" "$P/cell.c" "$P/comlist.c" "$P/dlist.c" "$P/ewald.c" \
    "$P/grid.c" "$P/iclist.c" "$P/nlist.c" "$P/pair_pot.c" "$P/slater.c" \
    "$P/tailcorr.c" "$P/truncation.c" "$P/vlist.c" -lm -o "$OUT/pes/ext$SUFFIX"
fi
# the checkout this extension was built from, for oracle/ref_shim.py
printf '%s\n' "$REF" > "$OUT/REFERENCE_ROOT"
echo "build_ref: $OUT/pes/ext$SUFFIX"
