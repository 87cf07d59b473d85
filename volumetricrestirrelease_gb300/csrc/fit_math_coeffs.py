import numpy as np
np.set_printoptions(precision=20)
def fit(f, lo, hi, basis_pows, n=20001, weight=None):
    # least-squares fit on Chebyshev-distributed nodes, relative error weighting
    k = np.arange(n)
    x = 0.5*(lo+hi) + 0.5*(hi-lo)*np.cos(np.pi*(k+0.5)/n)
    y = f(x)
    A = np.stack([x**p for p in basis_pows], axis=1)
    w = 1.0/np.abs(y) if weight is None else weight(x)
    c, *_ = np.linalg.lstsq(A*w[:,None], y*w, rcond=None)
    return c
# exp(r) on [-ln2/2, ln2/2]: 1 + r + c2 r^2 + ... + c7 r^7  (fit remainder)
L = np.log(2)/2
c = fit(lambda r: np.expm1(r)-r, -L, L, [2,3,4,5,6,7], weight=lambda r: 1/np.maximum(np.exp(r),1e-300))
print("exp", [float(np.float32(v)) for v in c])
# log: log(m) = 2 s (1 + a1 z + a2 z^2 + a3 z^3 + a4 z^4), s=(m-1)/(m+1), z=s^2 ; |s|<=0.1716
S = (np.sqrt(2)-1)/(np.sqrt(2)+1)
def g(z):
    s = np.sqrt(z); return np.arctanh(s)/s - 1
c = fit(g, 1e-12, S*S, [1,2,3,4], weight=lambda z: np.ones_like(z))
print("log", [float(np.float32(v)) for v in c])
# sin(r) = r + r^3 (s1 + s2 z + s3 z^2 + s4 z^3), z=r^2, r in [-pi/4, pi/4]
P4 = np.pi/4
c = fit(lambda z: (np.sin(np.sqrt(z)) - np.sqrt(z))/np.sqrt(z)**3, 1e-10, P4*P4, [0,1,2,3], weight=lambda z: np.ones_like(z))
print("sin", [float(np.float32(v)) for v in c])
# cos(r) = 1 - z/2 + z^2 (c1 + c2 z + c3 z^2 + c4 z^3)
c = fit(lambda z: (np.cos(np.sqrt(z)) - 1 + z/2)/z**2, 1e-6, P4*P4, [0,1,2,3], weight=lambda z: np.ones_like(z))
print("cos", [float(np.float32(v)) for v in c])
# atan(x) = x + x^3 (t1 + t2 z + ... t6 z^5) on [0, tan(pi/12)]
T = np.tan(np.pi/12)
c = fit(lambda z: (np.arctan(np.sqrt(z)) - np.sqrt(z))/np.sqrt(z)**3, 1e-10, T*T, [0,1,2,3,4], weight=lambda z: np.ones_like(z))
print("atan", [float(np.float32(v)) for v in c])
# splits
def split(v, bits):
    m, e = np.frexp(v); q = np.floor(m*2**bits)/2**bits; hi = np.ldexp(q, e); return hi
ln2 = np.log(2)
hi = split(ln2, 16); lo = np.float32(ln2 - hi); print("ln2", repr(float(np.float32(hi))), repr(float(lo)), float(np.float32(hi))==hi)
pio2 = np.pi/2
h1 = split(pio2, 12); r1 = pio2 - h1; h2 = split(r1, 12); r2 = r1 - h2; h3 = np.float32(r2)
print("pio2", repr(float(h1)), repr(float(h2)), repr(float(h3)))
