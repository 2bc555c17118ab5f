#!/bin/sh
# Builds the C oracle (test infrastructure) into oracle/_build/.
# The reference crate itself is Rust (no cargo/rustc in this image), so there is
# no oracle/_ref build: the oracle is this restatement, checked against scipy's
# dggev and the reference's own known-answer tests.
set -e
here=$(cd "$(dirname "$0")" && pwd)
mkdir -p "$here/_build"
${CC:-gcc} -O2 -Wall -Wextra -shared -fPIC -o "$here/_build/libjne_oracle.so" "$here/jne_oracle.c" -lm -lpthread
