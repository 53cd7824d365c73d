#!/usr/bin/env bash
# Builds the reference oracle oracle/_ref/libxmdref64.so from the reference's
# own hot-path translation units (TEST INFRASTRUCTURE; never shipped).
#
#   XMD_REF_ROOT   reference checkout (default /root/reference); its xmd/ tree
#                  is read, never written.  Exit status 2 when it is absent.
#
# The reference root used is recorded in oracle/_ref/ref_root.txt, where tests
# that read the reference's example data find it.
#
# The FP64 oracle is the reference with `using real = double;`
# (xmd/include/xmd/types/scalar.h:4).  The reference has no such switch, so the
# include tree is copied into oracle/_ref/fp64/ (git-ignored build output) and
# that one line is edited there.  Sources compile where they lie.  Boost is
# replaced by the empty stubs under oracle/ref/stub/ (only `access` and a few
# helper names are referenced), and `particle_pairs` is mapped to the
# non-native Verlet list, the list the shipped code names but never declares.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${XMD_REF_ROOT:-/root/reference}/xmd"
OUT="$HERE/../_ref"
if [ ! -d "$REF/src" ]; then
  echo "reference tree not found at $REF" >&2
  exit 2
fi
mkdir -p "$OUT/obj"
rm -rf "$OUT/fp64"
mkdir -p "$OUT/fp64"
cp -r "$REF/include" "$OUT/fp64/include"
sed -i 's/using real = float;/using real = double;/' "$OUT/fp64/include/xmd/types/scalar.h"
grep -q 'using real = double;' "$OUT/fp64/include/xmd/types/scalar.h"
# [D10] sync_diff_expr derives from sync_data_expr<sync_sum_expr<...>>
# (xmd/include/xmd/forces/qa/sync_data.h:107-108), so `sync - diff` evaluates
# as `sync + diff` and the QA valence checks of sift_candidates.cpp:60-73 and
# process_candidates.cpp:17-20 never bind.  The oracle uses the subtraction
# the code spells out: the CRTP base names the difference expression.
sed -i '/class sync_diff_expr:/{n;s/sync_data_expr<sync_sum_expr<E1, E2>>/sync_data_expr<sync_diff_expr<E1, E2>>/}' \
  "$OUT/fp64/include/xmd/forces/qa/sync_data.h"
grep -A1 'class sync_diff_expr:' "$OUT/fp64/include/xmd/forces/qa/sync_data.h" | grep -q 'sync_data_expr<sync_diff_expr<E1, E2>>'
INC=(-I"$OUT/fp64/include" -I"$OUT/fp64/include/xmd" -I"$REF/src"
     -I"$REF/ext/gentypes/include" -I"$REF/ext/yaml-cpp-0.7.0/include" -I"$REF/ext/eigen-3.4.0" -I"$HERE/stub")
FLAGS=(-std=c++17 -O2 -fPIC -Wno-changes-meaning -Dparticle_pairs=non_native)
TUS=(forces/tether forces/go forces/primitives/lj forces/primitives/sink_lj
     forces/primitives/harmonic forces/angle/native forces/dihedral/complex_native
     forces/dihedral/simple_native forces/pauli forces/es/const forces/es/relative
     forces/es/es_pair forces/qa/precompute_nh forces/qa/sift_candidates
     forces/qa/process_candidates forces/qa/process_contacts forces/qa/free_pair
     dynamics/lang_pc nl/verify forces/chiral forces/native_ss forces/angle/heurestic
     forces/dihedral/heurestic model/model forces/velocity_afm forces/force_afm forces/walls/solid forces/walls/lj_attr
     forces/pid/eval_forces forces/pid/bundle)
OBJS=()
pids=()
for tu in "${TUS[@]}"; do
  o="$OUT/obj/$(echo "$tu" | tr / _).o"
  OBJS+=("$o")
  g++ "${FLAGS[@]}" "${INC[@]}" -c "$REF/src/$tu.cpp" -o "$o" &
  pids+=($!)
done
g++ "${FLAGS[@]}" "${INC[@]}" -c "$HERE/ref_driver.cpp" -o "$OUT/obj/ref_driver.o" &
pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
g++ -shared -o "$OUT/libxmdref64.so" "${OBJS[@]}" "$OUT/obj/ref_driver.o"
echo "${XMD_REF_ROOT:-/root/reference}" > "$OUT/ref_root.txt"
echo "built $OUT/libxmdref64.so"
