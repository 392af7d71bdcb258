"""Restated Formura front end (parser, Orthotope Machine, Manifest Machine)
and the code emitters of the GB300 backend."""
