"""Build step: embed a source file in the library as a C string (the device
math header, compiled again at run time by the JIT path).

usage: python embed_src.py <input> <output.h> <symbol>
"""
import sys

src, out, sym = sys.argv[1:4]
text = open(src).read()
delim = "NT2G_SRC"
assert (")" + delim + '"') not in text
with open(out, "w") as f:
    f.write(f"// generated from {src.split('/')[-1]} by embed_src.py; do not edit\n")
    f.write(f'static const char {sym}[] = R"{delim}(\n{text}){delim}";\n')
