"""Embed the reference's LEMS core-component XML as a C byte array.

Test infrastructure for the oracle build only.  The reference embeds
eden/neuroml/LEMS_CoreComponents.inc.xml with `xxd -i` (reference Makefile,
the LEMS_CoreComponents object rule); xxd is not installed here, so this
script writes the same two symbols, `eden_neuroml_LEMS_CoreComponents_inc_xml`
and `eden_neuroml_LEMS_CoreComponents_inc_xml_len`, which
eden/NeuroML.cpp:9750-9751 reads.

usage: python embed_core_xml.py <input.xml> <output.cpp>
"""
import sys


def main(src: str, dst: str) -> None:
    data = open(src, "rb").read()
    lines = []
    for i in range(0, len(data), 16):
        lines.append("  " + ", ".join("0x%02x" % b for b in data[i:i + 16]) + ",")
    with open(dst, "w") as f:
        f.write("unsigned char eden_neuroml_LEMS_CoreComponents_inc_xml[] = {\n")
        f.write("\n".join(lines))
        f.write("\n};\n")
        f.write("unsigned int eden_neuroml_LEMS_CoreComponents_inc_xml_len = %d;\n" % len(data))


if __name__ == "__main__":
    main(sys.argv[1], sys.argv[2])
