"""Unit conversions and element tables (jrystal/_src/const.py:17-21)."""
BOHR2ANGSTROM = 0.529177249
ANGSTROM2BOHR = 1.8897259886
HARTREE2EV = 27.211386245988
EV2HARTREE = 1 / HARTREE2EV

_SYMBOLS = (
  "X H He Li Be B C N O F Ne Na Mg Al Si P S Cl Ar K Ca Sc Ti V Cr Mn Fe Co "
  "Ni Cu Zn Ga Ge As Se Br Kr Rb Sr Y Zr Nb Mo Tc Ru Rh Pd Ag Cd In Sn Sb Te "
  "I Xe Cs Ba La Ce Pr Nd Pm Sm Eu Gd Tb Dy Ho Er Tm Yb Lu Hf Ta W Re Os Ir "
  "Pt Au Hg Tl Pb Bi Po At Rn"
).split()
SYMBOL_TO_Z = {s: i for i, s in enumerate(_SYMBOLS) if i > 0}
Z_TO_SYMBOL = {i: s for s, i in SYMBOL_TO_Z.items()}


def fft_sizes(limit: int = 2048):
  """Sizes 2^a 3^b 5^c 7^d up to ``limit`` (the FFT-size table that
  jrystal/_src/const.py:265 lists)."""
  out = set()
  p2 = 1
  while p2 <= limit:
    p3 = p2
    while p3 <= limit:
      p5 = p3
      while p5 <= limit:
        p7 = p5
        while p7 <= limit:
          out.add(p7)
          p7 *= 7
        p5 *= 5
      p3 *= 3
    p2 *= 2
  return sorted(out)


CUFFT_FACTORS = fft_sizes()
