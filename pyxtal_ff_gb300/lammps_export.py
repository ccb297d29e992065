"""LAMMPS ML-IAP export of a trained potential: the text files the reference writes
next to its checkpoints (NN: pyxtal_ff/models/neuralnetwork.py:719-836, linear:
pyxtal_ff/models/polynomialregression.py:286-345) and that LAMMPS' ML-IAP
``nn`` / ``linear`` models with the ``sna`` descriptor read.

The files are an on-disk format, so the layout is byte-for-byte the reference's:
- ``NN_weights.txt``: the species count and the parameter count of the last network,
  the ``NET`` line (descriptor count, layer count, per layer its lower-cased
  activation and width), then per element the drange offsets (``# Scale0``: dmin)
  and widths (``# Scale1``: dmax - dmin), five per line in %20.13f, and the layer
  coefficients row by row, each row its bias then its weights, five per line in
  %18.13f;
- ``PR_weights.txt``: the species count, d_max + 1, then the coefficients one per line;
- ``DescriptorParam.txt``: rcutfac, twojmax (= 2 lmax), the elements, and for SNAP
  radelems (0.5 each), welems (the SNAP weights), rfac0, rmin0 0, switchflag 1,
  bzeroflag 0.
"""
from __future__ import annotations

import numpy as np


def network_layout(net):
    """(layer widths incl. the output, activation names per layer, [(weight, bias)]) of
    a torch Sequential of Linear layers each optionally followed by an activation
    module; a Linear not followed by one has activation 'Linear'."""
    import torch
    mods = list(net.children()) if isinstance(net, torch.nn.Sequential) else list(net.modules())[1:]
    widths, acts, params = [], [], []
    for i, m in enumerate(mods):
        if isinstance(m, torch.nn.Linear):
            widths.append(m.out_features)
            params.append((m.weight.detach().cpu().double().numpy(), m.bias.detach().cpu().double().numpy()))
            nxt = mods[i + 1] if i + 1 < len(mods) else None
            acts.append("Linear" if nxt is None or isinstance(nxt, torch.nn.Linear) else type(nxt).__name__)
    return widths, acts, params


def _rows5(values, fmt):
    """values in fmt, each followed by a space, a newline after every fifth and after the last."""
    out = []
    n = len(values)
    for i, v in enumerate(values, start=1):
        out.append(fmt.format(v) + " ")
        if i % 5 == 0 or i == n:
            out.append("\n")
    return "".join(out)


def nn_weights_text(elements, models, drange, no_of_descriptors):
    elements = sorted(elements)
    layouts = {e: network_layout(models[e]) for e in elements}
    nparams = 0
    for w, b in layouts[elements[-1]][2]:
        nparams += w.size + b.size
    s = ["# Neural networks weights generated in PyXtal_FF \n", "# total_species nparams \n",
         f"{len(elements)} ", f"{nparams} \n\n"]
    for n, e in enumerate(elements):
        widths, acts, params = layouts[e]
        if n == 0:
            s.append("# NET ndescriptors nlayers activation_func for layer 1, number of nodes for layer 1, ..., ..., "
                     "...., \n")
            s.append(f"NET {no_of_descriptors} {len(widths)} ")
            for a, h in zip(acts, widths):
                s.append(f"{a} ".lower())
                s.append(f"{h} ")
        s.append("\n\n")
        dr = np.asarray(drange[e], dtype=np.float64)
        s.append("# Scale0 \n")
        s.append(_rows5(dr[:, 0], "{:20.13f}"))
        s.append("\n")
        s.append("# Scale1 \n")
        s.append(_rows5(dr[:, 1] - dr[:, 0], "{:20.13f}"))
        s.append("\n")
        s.append("# Coefficients ({:s})\n".format(e))
        cnt = 1
        for w, b in params:
            for row in np.concatenate([b[:, None], w], axis=1):
                for v in row:
                    s.append("{:18.13f} \n".format(v) if cnt % 5 == 0 else "{:18.13f} ".format(v))
                    cnt += 1
        s.append("\n" if (cnt - 1) % 5 == 0 else "\n\n")
    return "".join(s)


def pr_weights_text(elements, coef_, d_max):
    s = ["# Polynomial Regression weights generated in PyXtal_FF \n", "# total_species ncoefficient \n\n",
         f"{len(elements)} {d_max + 1} \n"]
    count = 0
    for _ in sorted(elements):
        for _ in range(d_max + 1):
            s.append(f"{coef_[count]} \n")
            count += 1
    return "".join(s)


def descriptor_param_text(elements, des_info):
    elements = sorted(elements)
    t = des_info["type"]
    s = ["# Descriptor parameters generated in PyXtal_FF \n\n", "# Required \n", f"rcutfac {des_info['Rc']} \n"]
    if t in ("SO3", "SOAP"):
        raise NotImplementedError("SO3 descriptors are not part of this path")
    s.append(f"twojmax {des_info['parameters']['lmax'] * 2} \n\n")
    s.append("# Elements \n\n")
    s.append(f"nelems {len(elements)} \n")
    s.append("elems " + "".join(f"{e} " for e in elements) + "\n")
    if t in ("snap", "SNAP"):
        s.append("radelems " + "0.5 " * len(elements) + "\n")
        s.append("welems " + "".join(f"{des_info['weights'][e]} " for e in elements) + "\n\n")
        s.append(f"rfac0 {des_info['parameters']['rfac']} \n")
        s.append("rmin0 0 \n")
        s.append("switchflag 1 \n")
        s.append("bzeroflag 0 \n")
    return "".join(s)


def write_nn(path, elements, models, drange, no_of_descriptors, des_info):
    """NN_weights.txt and DescriptorParam.txt under the prefix `path` (as the reference
    joins self.path + name)."""
    with open(path + "NN_weights.txt", "w") as f:
        f.write(nn_weights_text(elements, models, drange, no_of_descriptors))
    with open(path + "DescriptorParam.txt", "w") as f:
        f.write(descriptor_param_text(elements, des_info))


def write_pr(path, elements, coef_, d_max, des_info):
    """PR_weights.txt and DescriptorParam.txt under the prefix `path`."""
    with open(path + "PR_weights.txt", "w") as f:
        f.write(pr_weights_text(elements, coef_, d_max))
    with open(path + "DescriptorParam.txt", "w") as f:
        f.write(descriptor_param_text(elements, des_info))
