"""Physical constants of the reference (bin/globals.h:4-16), SI units."""
PI = 3.14159265358979323
EL_CHARGE = 1.60217733e-19   # C
AMU = 1.6605402e-27          # kg
KE = 8.987551787e9           # 1/(4 pi eps0), N m^2 / C^2
KB = 1.3806504e-23           # J/K
EV_TO_JOULE = 1.60217646e-19
