set output "hist_group1_MOTIF00000.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-71.1796:25.4054]
set yrange [0:197656]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_group1_MOTIF00000.dat" using 1:2 title 'MOTIF00000 (group1)' with boxes
