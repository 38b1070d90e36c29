"""Input formats feeding the encoder: the reference's character-matrix and
prior readers (laml_libs/sequence_lib.py:100-363) and writer (78-92).

``read_sequences`` returns (charMtrx, site_names) with charMtrx =
{cell: [int | '?']}; ``read_priors`` returns Q = [{state: prob}] per site
(CSV ``site,state,prob`` with an optional header and optional 'r'-prefixed
site names, or a pickled {site: {state: prob}} dict where state 0 gets prior
0).  These feed ``problem.dataset_from_rows`` / ``fastEM_solver``.
"""
from __future__ import annotations

import pickle
from typing import Dict, List, Optional, Sequence, Tuple

RECOGNIZED_MISSING = {"-", "?", "-1"}   # sequence_lib.py:8


def _is_missing(seen, x):
    if x in seen or x in RECOGNIZED_MISSING or x.isalpha():
        return True
    try:
        return int(x) < 0
    except ValueError:
        return False


def read_char_matrix(path: str, delimiter: str = ",", masked_symbol: Optional[str] = None,
                     replace_mchar: str = "?") -> Tuple[Dict[str, list], List[str]]:
    """sequence_lib.read_charMtrx (sequence_lib.py:139-175)."""
    seen = {masked_symbol} if masked_symbol is not None else set()
    D = {}
    with open(path) as f:
        site_names = f.readline().strip().split(delimiter)
        if site_names[0] == "cell_name" or "cell" in site_names[0]:
            site_names = site_names[1:]
        for line in f:
            parts = line.strip().split(delimiter)
            if len(parts) < 2:
                continue
            seq = []
            for x in parts[1:]:
                if _is_missing(seen, x):
                    seen.add(x)
                    seq.append(replace_mchar if replace_mchar is not None else x)
                else:
                    seq.append(int(x))
            D[parts[0]] = seq
    return D, site_names


def read_sequences(path: str, filetype: str = "charMtrx", delimiter: str = ",",
                   masked_symbol: Optional[str] = None, suppress_warnings: bool = False,
                   replace_mchar: str = "?"):
    if filetype != "charMtrx":
        raise ValueError("only the charMtrx format is supported")
    return read_char_matrix(path, delimiter, masked_symbol, replace_mchar)


def read_priors(path: str, msa: Optional[dict] = None,
                site_names: Optional[Sequence[str]] = None) -> List[Dict[int, float]]:
    """sequence_lib.read_priors: CSV (324-355) or pickle (261-322, the
    site-name matching branch excepted: keys are taken in sorted order)."""
    ext = path.strip().split(".")[-1]
    if ext in ("pkl", "pickle"):
        with open(path, "rb") as f:
            priors = pickle.load(f)
        Q = []
        for i in sorted(priors.keys()):
            q = {int(x): priors[i][x] for x in priors[i]}
            q[0] = 0
            Q.append(q)
        return Q
    Q, Qi, seen = [], {}, set()
    with open(path) as f:
        lines = f.readlines()
    tokens = lines[0].split(",")
    if not tokens[1].isnumeric() and not tokens[2].isnumeric():
        lines = lines[1:]
    charname_is_str = not lines[0].split(",")[0].isnumeric()
    for line in lines:
        site, state, prob = line.strip().split(",")
        site = int(site[1:]) if charname_is_str else int(site)
        if site not in seen:
            if seen:
                Q.append(Qi)
                Qi = {}
            seen.add(site)
        Qi[int(state)] = float(prob)
    Q.append(Qi)
    return Q


def write_sequences(char_mtrx: dict, nsites: int, path: str, delimiter: str = ","):
    """sequence_lib.write_sequences (sequence_lib.py:78-92)."""
    with open(path, "w") as f:
        f.write("cell" + "".join(delimiter + "r" + str(i) for i in range(nsites)) + "\n")
        for cell, seq in char_mtrx.items():
            f.write(cell + "".join(delimiter + str(x) for x in seq) + "\n")
