"""C source that prints sizeof/offsetof of the three public structs as JSON."""
import qssgpu as Q

STRUCTS = {"Grid": Q.Grid, "QSS_DataArrays": Q.QSSDataArrays, "Options": Q.Options}


def probe_source(header: str) -> str:
    lines = [header, "#include <stdio.h>", "#include <stddef.h>", "int main(void){", 'printf("{");']
    first = True
    for cname, cls in STRUCTS.items():
        entries = [(f"{cname}.sizeof", f"sizeof({cname})")]
        entries += [(f"{cname}.{f[0]}", f"offsetof({cname}, {f[0]})") for f in cls._fields_]
        for key, expr in entries:
            sep = "" if first else ","
            first = False
            lines.append(f'printf("{sep}\\"{key}\\": %zu", (size_t)({expr}));')
    lines += ['printf("}\\n");', "return 0;}"]
    return "\n".join(lines)
