# A 9-point star in four dimensions written with loops in the stencil language: centre weight
# A, then for each axis 0..3 the +1 and -1 neighbours with weight B.  Axis 0 is contiguous.
from st.expr import Index, ConstRef
from st.grid import Grid

ax = [Index(n) for n in range(4)]
src = Grid("u", 4)
dst = Grid("v", 4)

acc = ConstRef("A") * src(*ax)
for a in range(4):
    for s in (1, -1):
        idx = list(ax)
        idx[a] = ax[a] + s
        acc = acc + ConstRef("B") * src(*idx)
dst(*ax).assign(acc)
STENCIL = [dst]
