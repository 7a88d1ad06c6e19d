# A 13-point star written with loops in the stencil language (taps: centre, then the
# rings at distance 1 and 2 in the order +i -i +j -j +k -k), coefficients W0, W1, W2.
from st.expr import Index, ConstRef
from st.grid import Grid

ax = [Index(0), Index(1), Index(2)]
src = Grid("u", 3)
dst = Grid("v", 3)
w = [ConstRef("W0"), ConstRef("W1"), ConstRef("W2")]

acc = w[0] * src(*ax)
for d in (1, 2):
    for a in range(3):
        for s in (d, -d):
            idx = list(ax)
            idx[a] = ax[a] + s
            acc = acc + w[d] * src(*idx)
dst(*ax).assign(acc)
STENCIL = [dst]
