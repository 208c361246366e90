#!/bin/sh
# Builds the oracle (test infrastructure) into oracle/_build/liboracle.so.
set -e
cd "$(dirname "$0")"
mkdir -p _build
${CXX:-g++} -std=c++17 -O2 -fPIC -shared -ffp-contract=off -Wall -Wno-unused-function \
  -o _build/liboracle.so oracle.cpp -lpthread
