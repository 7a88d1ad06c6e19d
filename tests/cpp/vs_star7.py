# A 7-point star in the reference's stencil language, one coefficient per tap read from the
# caller's `coeff` array (the tap order of stencils/3axis.cpp's arr_func: centre, i+1, i-1,
# j+1, j-1, k+1, k-1).  Used by vs_bricks.cpp through a brick(...) statement.
from st.expr import Index, ConstRef
from st.grid import Grid

i, j, k = Index(0), Index(1), Index(2)
src = Grid("bIn", 3)
dst = Grid("bOut", 3)
taps = [(0, 0, 0), (1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)]
total = None
for n, (di, dj, dk) in enumerate(taps):
    term = ConstRef("coeff[%d]" % n) * src(i + di, j + dj, k + dk)
    total = term if total is None else total + term
dst(i, j, k).assign(total)
STENCIL = [dst]
