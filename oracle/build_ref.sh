#!/usr/bin/env bash
# Build the unmodified reference CSEM solver from its sources, where they lie, into
# oracle/_ref/ (git-ignored). Test infrastructure only: the result is the CPU oracle
# that pins oracle/csem_oracle.c and generates tests/golden fixtures.
#
#   REF=<reference checkout> oracle/build_ref.sh
#
# REF defaults to CSEM_REFERENCE_DIR, else to a sibling directory "reference" of this
# repository.
#
# Sources: every reference .c except Acoo.c (MUMPS direct solver, reached only from the
# dead main3 in main.c:226-280; MUMPS is not installed). MPI and FFTW are replaced by
# oracle/ref_stubs (one-rank MPI, self-written DFT). main.c is compiled with
# -Dmain=ref_main so the driver can also be called from the harness.
# Flags follow the reference Makefile (-O3), plus -ffp-contract=off so that builds on
# aarch64 (where GCC would otherwise fuse multiply-adds) match x86-64 bit for bit.
# REF_VARIANT=fma builds instead into oracle/_ref_fma/ with multiply-add contraction
# (-ffp-contract=fast, plus -mfma on x86-64): what the reference Makefile's flags give on
# aarch64, used to measure how far the reference's own results move between builds.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${REF:-${CSEM_REFERENCE_DIR:-$(cd "$HERE/../.." && pwd)/reference}}"
CONTRACT="-ffp-contract=off"
OUT="$HERE/_ref"
if [ "${REF_VARIANT:-}" = "fma" ]; then
  CONTRACT="-ffp-contract=fast"
  if [ "$(uname -m)" = "x86_64" ]; then CONTRACT="$CONTRACT -mfma"; fi
  OUT="$HERE/_ref_fma"
fi
OBJ="$OUT/obj"
if [ ! -f "$REF/fdfd.c" ]; then
  echo "build_ref.sh: reference sources not found at $REF" >&2
  exit 2
fi
mkdir -p "$OBJ"
CC="${CC:-gcc}"
CFLAGS="-O3 -fPIC $CONTRACT -w -std=gnu99"
INC="-I$HERE/ref_stubs -I$REF"
SRCS="cstd.c emf_init_free.c acq_init_free.c extend_model.c create_nugrid.c find_index.c \
      fdfd.c airbc_init_free.c inject_extract.c solver.c cdotprod.c gmres_init_free.c \
      write_data.c Acsr.c"
pids=()
for s in $SRCS; do
  $CC $CFLAGS $INC -c "$REF/$s" -o "$OBJ/${s%.c}.o" & pids+=($!)
done
$CC $CFLAGS $INC -Dmain=ref_main -c "$REF/main.c" -o "$OBJ/main.o" & pids+=($!)
$CC $CFLAGS $INC -c "$HERE/ref_stubs/ref_stubs.c" -o "$OBJ/ref_stubs.o" & pids+=($!)
$CC $CFLAGS $INC -c "$HERE/ref_stubs/ref_harness.c" -o "$OBJ/ref_harness.o" & pids+=($!)
$CC $CFLAGS -c "$HERE/fft2d.c" -o "$OBJ/fft2d.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
$CC -shared -o "$OUT/libcsemref.so" "$OBJ"/*.o -lm
# a stand-alone reference executable (same objects, ref_main as entry point)
cat > "$OBJ/exe_main.c" <<'EOF'
int ref_main(int argc, char **argv);
int main(int argc, char **argv) { return ref_main(argc, argv); }
EOF
$CC $CFLAGS -c "$OBJ/exe_main.c" -o "$OBJ/exe_main.o.x"
$CC -o "$OUT/csem_ref_main" "$OBJ/exe_main.o.x" $(ls "$OBJ"/*.o | grep -v ref_harness) -lm
echo "built $OUT/libcsemref.so and $OUT/csem_ref_main"
