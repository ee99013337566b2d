set output "hist_group2_MOTIF00000.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-72.0947:24.6021]
set yrange [0:192244]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_group2_MOTIF00000.dat" using 1:2 title 'MOTIF00000 (group2)' with boxes
