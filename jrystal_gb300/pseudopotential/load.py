"""UPF (Unified Pseudopotential Format, v2 XML) reader
(jrystal/pseudopotential/load.py:27-241).

Only the sections the norm-conserving energy path reads are interpreted:
PP_HEADER attributes, PP_MESH (PP_R, PP_RAB), PP_LOCAL, PP_NONLOCAL
(PP_BETA.i with their attributes, PP_DIJ, and PP_AUGMENTATION when present)
and PP_INFO's valence-configuration table.  The returned dictionary has the
reference's keys, so code written against jrystal's parse_upf reads it
unchanged.
"""
from __future__ import annotations

import os
import xml.etree.ElementTree as ET
from typing import Dict, List

_TRUE = ("true", "True", "T", "t", "1", "TRUE")


def _floats(text) -> List[float]:
  return [float(v) for v in (text or "").split()]


def _after_colon(line: str) -> str:
  head, sep, tail = line.partition(":")
  return tail.strip() if sep else line.strip()


def parse_valence_configuration(lines) -> List[dict]:
  """Rows 'nl pn l occ Rcut Rcut_US E_pseu' of PP_INFO's valence table."""
  out = []
  for line in lines:
    parts = line.split()
    if len(parts) < 7 or parts[0] == "nl" or line.lstrip().lower().startswith("generation"):
      continue
    try:
      out.append({"nl": parts[0], "pn": int(parts[1]), "l": int(parts[2]), "occ": float(parts[3]),
                  "Rcut": float(parts[4]), "Rcut_US": float(parts[5]), "E_pseu": float(parts[6])})
    except ValueError:
      continue
  return out


def parse_pp_info(text: str) -> Dict:
  """PP_INFO as a dictionary: the first ten lines by position (generator,
  author, date, type, element, functional, suggested cutoffs, relativistic
  flag, local-potential line) and the valence-configuration table."""
  lines = text.split("\n")
  get = lambda i: _after_colon(lines[i]) if i < len(lines) else ""
  start = end = None
  for i, line in enumerate(lines):
    low = line.lower()
    if start is None and "valence configuration" in low:
      start = i
    elif start is not None and "generation configuration" in low:
      end = i
      break
  valence = parse_valence_configuration(lines[start + 1:end]) if start is not None else []
  return {
    "Generated by": get(0), "Author": get(1), "Generation date": get(2),
    "Pseudopotential type": get(3), "Element": get(4), "Functional": get(5),
    "Suggested minimum cutoff for wavefunctions": get(6),
    "Suggested minimum cutoff for charge density": get(7),
    "Relativistic Calculation": lines[8].strip() if len(lines) > 8 else "",
    "Local Potential": get(9),
    "Valence configuration": valence,
    "Generation configuration": lines[-1].strip() if lines else "",
  }


def parse_pp_nonlocal(node) -> Dict:
  out: Dict = {}
  betas = [e for e in node if e.tag.startswith("PP_BETA")] if node is not None else []
  if betas:
    out["PP_BETA"] = [{
      "index": b.get("index"), "label": b.get("label"),
      "angular_momentum": b.get("angular_momentum"),
      "cutoff_radius_index": b.get("cutoff_radius_index"),
      "cutoff_radius": b.get("cutoff_radius"),
      "ultrasoft_cutoff_radius": b.get("ultrasoft_cutoff_radius"),
      "values": _floats(b.text)} for b in betas]
  if node is not None and node.find("PP_DIJ") is not None:
    out["PP_DIJ"] = _floats(node.find("PP_DIJ").text)
  aug = node.find("PP_AUGMENTATION") if node is not None else None
  if aug is not None:
    a = {"q_with_l": aug.get("q_with_l") in _TRUE, "nqf": int(aug.get("nqf", 0)),
         "nqlc": int(aug.get("nqlc", 0))}
    if aug.find("PP_Q") is not None:
      a["PP_Q"] = _floats(aug.find("PP_Q").text)
    qij = [e for e in aug if e.tag.startswith("PP_QIJ")]
    if qij:
      a["PP_QIJ"] = [{"first_index": q.get("first_index"), "second_index": q.get("second_index"),
                      "composite_index": q.get("composite_index"),
                      "angular_momentum": q.get("angular_momentum"),
                      "values": _floats(q.text)} for q in qij]
    out["PP_AUGMENTATION"] = a
  return out


def parse_upf(filepath: str) -> Dict:
  """Sections of a UPF v2 file: PP_INFO, PP_HEADER, PP_MESH, PP_NONLOCAL,
  PP_LOCAL (values in the file's Rydberg units)."""
  root = ET.parse(filepath).getroot()
  info = root.find("PP_INFO")
  mesh = root.find("PP_MESH")
  header = root.find("PP_HEADER")
  if header is None or mesh is None or root.find("PP_LOCAL") is None:
    raise ValueError(f"{filepath}: not a UPF v2 file (PP_HEADER, PP_MESH and PP_LOCAL are required)")
  return {
    "PP_INFO": parse_pp_info((info.text or "").strip() if info is not None else ""),
    "PP_HEADER": dict(header.attrib),
    "PP_MESH": {"info": dict(mesh.attrib), "PP_R": _floats(mesh.find("PP_R").text),
                "PP_RAB": _floats(mesh.find("PP_RAB").text)},
    "PP_NONLOCAL": parse_pp_nonlocal(root.find("PP_NONLOCAL")),
    "PP_LOCAL": _floats(root.find("PP_LOCAL").text),
  }


def find_upf(dir_path: str, atom: str) -> str:
  """The file of ``atom`` in ``dir_path``: a name starting with '<symbol>.'
  and ending in 'upf', case-insensitive (load.py:219-241)."""
  for name in sorted(os.listdir(dir_path)):
    low = name.lower()
    if low.startswith(atom.lower() + ".") and low.endswith("upf"):
      return os.path.join(dir_path, name)
  raise ValueError(f"The pseudopotential file of element '{atom}' is not found in directory "
                   f"{dir_path}")
