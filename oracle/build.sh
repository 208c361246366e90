#!/bin/sh
# Builds the oracle (test infrastructure) into oracle/_build:
#   liboracle.so           FP expressions evaluated as written (no contraction),
#                          the arithmetic of the reference built for x86-64;
#   liboracle_contract.so  multiply-adds contracted into FMAs, the arithmetic
#                          of the reference built by gcc for aarch64 (its
#                          default -ffp-contract=fast). Tests use it only to
#                          tell whether a pair's result depends on rounding.
set -e
cd "$(dirname "$0")"
mkdir -p _build
FMA=""
case "$(uname -m)" in x86_64|amd64) FMA="-mfma" ;; esac
${CXX:-g++} -std=c++17 -O2 -fPIC -shared -ffp-contract=off -Wall -Wno-unused-function \
  -o _build/liboracle.so oracle.cpp -lpthread &
plain=$!
${CXX:-g++} -std=c++17 -O2 -fPIC -shared -ffp-contract=fast $FMA -Wall -Wno-unused-function \
  -o _build/liboracle_contract.so oracle.cpp -lpthread &
contract=$!
rc=0
wait $plain || rc=1
wait $contract || rc=1
exit $rc
