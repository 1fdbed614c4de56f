#!/bin/sh
# Compiles the reference muFFT library from its own sources into
# oracle/_ref/libmufft_ref.so (test infrastructure only: golden-vector
# generation and CPU-side parity of the oracle restatement).  The reference's CMake build is
# not used; this is the same set of translation units and per-file ISA flags
# (CMakeLists.txt:23-63) driven by gcc directly.  Nothing is copied: the
# sources are read where they lie.
#
# usage: oracle/build_ref.sh reference_dir [output_dir]
set -eu
if [ $# -lt 1 ]; then
    echo "usage: $0 reference_dir [output_dir]" >&2
    exit 2
fi
REF=$1
OUT=${2:-$(dirname "$0")/_ref}
CC=${CC:-gcc}
if [ ! -f "$REF/fft.c" ]; then
    echo "build_ref.sh: reference sources not found at $REF" >&2
    exit 2
fi
mkdir -p "$OUT/obj"
CFLAGS="-std=gnu99 -O2 -fPIC -ffp-contract=off -I$REF"
OBJS=""
case "$(uname -m)" in
    x86_64|amd64|i?86)
        DEFS="-DMUFFT_HAVE_X86 -DMUFFT_HAVE_SSE -DMUFFT_HAVE_SSE3 -DMUFFT_HAVE_AVX"
        $CC $CFLAGS -msse -mno-sse3 -mno-avx -c "$REF/x86/kernel.sse.c" -o "$OUT/obj/kernel_sse.o"
        $CC $CFLAGS -msse -msse3 -mno-avx -c "$REF/x86/kernel.sse3.c" -o "$OUT/obj/kernel_sse3.o"
        $CC $CFLAGS -msse -msse3 -mavx -c "$REF/x86/kernel.avx.c" -o "$OUT/obj/kernel_avx.o"
        OBJS="$OUT/obj/kernel_sse.o $OUT/obj/kernel_sse3.o $OUT/obj/kernel_avx.o"
        ;;
    *)
        DEFS=""
        ;;
esac
for f in fft kernel cpu; do
    $CC $CFLAGS $DEFS -c "$REF/$f.c" -o "$OUT/obj/$f.o"
    OBJS="$OBJS $OUT/obj/$f.o"
done
$CC -shared -Wl,-Bsymbolic -o "$OUT/libmufft_ref.so" $OBJS -lm
echo "built $OUT/libmufft_ref.so"
