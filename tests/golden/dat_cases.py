"""The .dat description cases shared by make_dat_golden.py and tests/test_formats.py.

Each case: the .dat text, and the raw files (name -> byte count) created next to it."""

CASES = [
    ("float3", "ObjectFileName: vol.raw\nResolution: 4 3 2\nSliceThickness: 1 1 2\nFormat: FLOAT3\n",
     {"vol.raw": 4 * 3 * 2 * 3 * 4}),
    ("uchar3_comments_crlf", "# a comment\r\nObjectFileName:\tv8.raw\r\nTaggedFileName: ignored\r\n"
     "Resolution: 5 4 3\r\nSliceThickness: 0.5 0.25 1.5\r\nFormat: UCHAR3\r\n", {"v8.raw": 5 * 4 * 3 * 3}),
    ("octal_and_hex_resolution", "ObjectFileName: o.raw\nResolution: 010 0x4 2\nFormat: UCHAR3\n",
     {"o.raw": 8 * 4 * 2 * 3}),
    ("timesteps", "ObjectFileName: ts%02d.raw\nResolution: 2 2 2\nFormat: FLOAT3\nTimeDependent: 0 2\n",
     {"ts00.raw": 96, "ts01.raw": 96, "ts02.raw": 96}),
    ("timesteps_offset", "ObjectFileName: t_%d.raw\nResolution: 2 2 2\nFormat: UCHAR3\nTimeDependent: 3 4\n",
     {"t_3.raw": 24, "t_4.raw": 24}),
    ("ushort_scalar", "ObjectFileName: s.raw\nResolution: 3 3 3\nFormat: USHORT\n", {"s.raw": 54}),
    ("format_trailing_text", "ObjectFileName: f.raw\nResolution: 2 2 2\nFormat: FLOAT   3 components\n",
     {"f.raw": 96}),
    ("format_no_digit", "ObjectFileName: g.raw\nResolution: 2 2 2\nFormat:    FLOAT\n", {"g.raw": 32}),
    ("spaces_and_order", "Format: UCHAR3\n   SliceThickness :  1e-1 2.5 3\nResolution:2 3 4\n"
     "   ObjectFileName   :   sp.raw   trailing\n", {"sp.raw": 2 * 3 * 4 * 3}),
    ("key_precedence", "ObjectFileName: Format.raw\nResolution: 2 2 2\nFormat: UCHAR3\n", {"Format.raw": 24}),
    ("commented_key", "#ObjectFileName: nope.raw\nObjectFileName: yes.raw\nResolution: 2 2 2\nFormat: UCHAR3\n",
     {"yes.raw": 24}),
    ("unknown_format", "ObjectFileName: u.raw\nResolution: 2 2 2\nFormat: DOUBLE3\n", {"u.raw": 1}),
    ("bad_timesteps", "ObjectFileName: b%d.raw\nResolution: 2 2 2\nFormat: UCHAR3\nTimeDependent: 3 1\n",
     {"b3.raw": 24}),
    ("short_resolution", "ObjectFileName: r.raw\nResolution: 4 4\nFormat: UCHAR3\n", {"r.raw": 48}),
    ("missing_colon", "ObjectFileName vol.raw\nResolution: 2 2 2\nFormat: UCHAR3\n", {"vol.raw": 24}),
    ("missing_raw", "ObjectFileName: absent.raw\nResolution: 2 2 2\nFormat: UCHAR3\n", {}),
    ("missing_timestep", "ObjectFileName: m%d.raw\nResolution: 2 2 2\nFormat: UCHAR3\nTimeDependent: 0 2\n",
     {"m0.raw": 24, "m1.raw": 24}),
]


def make_case(root, name, text, raws):
    """Write case `name` under root/name; returns the .dat path."""
    import os

    d = os.path.join(root, name)
    os.makedirs(d, exist_ok=True)
    for raw, n in raws.items():
        with open(os.path.join(d, raw), "wb") as fh:
            fh.write(bytes((i * 37 + 11) & 0xFF for i in range(n)))
    p = os.path.join(d, "case.dat")
    with open(p, "w", newline="") as fh:
        fh.write(text)
    return p
