#!/bin/sh
# build_ref.sh - compile the reference's own CPU join programs from their
# sources (read in place, never copied) into oracle/_ref/.  TEST
# INFRASTRUCTURE ONLY: the binaries pin the oracle to the reference's output
# (tests/golden/make_golden.py).  Needs the reference checkout; does nothing
# without it.  Outputs only into oracle/_ref/.
#
#   oracle/_ref/join_ori_{bnlj,hj,inner,outer}   joins/join_ori/*.cc as written
#                                                (read files R and S in the CWD)
#   oracle/_ref/{hash,inner,sortindex,block}_cpu joins/CPU_JOIN/*/ with
#                                                oracle/ref_shim.cpp injecting inputs
#   oracle/_ref/dist3_cpu, dist2_cpu             the distance joins joins/CPU_JOIN/3d_cpu
#                                                and joins/blockJoin_gpu/complex_block/2d_cpu,
#                                                the same way
set -e
REF=${EJ_REFERENCE:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -d "$REF/joins" ]; then
  echo "build_ref.sh: no reference at $REF, nothing built" >&2
  exit 0
fi
mkdir -p "$OUT"
CXX=${CXX:-g++}
# -ffp-contract=off: double arithmetic rounds each operation, as the reference's
# own x86-64 builds do (no fused multiply-add there)
FLAGS="-O2 -w -ffp-contract=off"

J="$REF/joins/join_ori"
$CXX $FLAGS -I"$J" "$J/bnlj.cc" -o "$OUT/join_ori_bnlj"
$CXX $FLAGS -I"$J" "$J/hj.cc" -o "$OUT/join_ori_hj"
$CXX $FLAGS -I"$J" "$J/inner-idx-bnlj.cc" -o "$OUT/join_ori_inner"
$CXX $FLAGS -I"$J" "$J/outer-idx-bnlj.cc" -o "$OUT/join_ori_outer"

C="$REF/joins/CPU_JOIN"
# name source-dir source-file right-global left-global result-global [shim defines]
shim() {
  $CXX $FLAGS -c -include "$HERE/ref_prelude.h" -I"$2" "$2/$3" -o "$OUT/$1.ref.o"
  $CXX $FLAGS -c -DEJ_REF_RIGHT="$4" -DEJ_REF_LEFT="$5" ${6:+-DEJ_REF_RESULT=$6} $7 "$HERE/ref_shim.cpp" \
    -o "$OUT/$1.shim.o"
  $CXX "$OUT/$1.ref.o" "$OUT/$1.shim.o" -o "$OUT/$1" -lm -lpthread
  rm -f "$OUT/$1.ref.o" "$OUT/$1.shim.o"
}
shim hash_cpu "$C/hash_cpu" hj.cc rt lt
shim inner_cpu "$C/inner_cpu" inner-idx-bnlj.cc rt lt jt
shim sortindex_cpu "$C/sortIndex_cpu" inner-idx-bnlj.cc rt lt jt
shim block_cpu "$C/block_cpu" nestLoopJoin.cc Tright Tleft Tjoin
shim dist3_cpu "$C/3d_cpu" nestLoopJoin.cc Tright Tleft Tjoin "-DEJ_REF_TUPLE_BYTES=32 -DEJ_REF_ROW_BYTES=56"
shim dist2_cpu "$REF/joins/blockJoin_gpu/complex_block/2d_cpu" nestLoopJoin.cc Tright Tleft Tjoin \
  "-DEJ_REF_TUPLE_BYTES=24 -DEJ_REF_ROW_BYTES=40"
echo "built reference programs into $OUT"
