# Domain Description 1.1

Interfaces 3

Interface: "cortex.1.tri"
Interface: "skull.1.tri"
Interface: "scalp.1.tri"

Domains 4

Domain Scalp: 2 -3
Domain Brain: -1
Domain Air: 3
Domain Skull: 1 -2
